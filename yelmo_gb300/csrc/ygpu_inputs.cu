// ygpu_inputs.cu -- the fields calc_ydyn derives before the velocity solve,
// and the SSA masks, on the GPU. Compiled with -fmad=false: the flotation
// test and every mask are evaluated exactly as written, in FP64, so they are
// bit-identical to a CPU evaluation of the same expressions.
#include <cuda_runtime.h>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

enum { MF_ICE_FREE = -1, MF_ICE_FREE_LAND = -2, MF_NONE = 0, MF_FLOAT = 1, MF_MARINE = 2, MF_GRND = 3 };

// calc_H_grnd (topography.f90:876-931, use_f_ice=.FALSE.), calc_z_srf_max
// (:820-849, binary f_ice), f_grnd of calc_f_grnd_subgrid_linear (:977-1105)
__global__ void k_inputs_pointwise(int n2, const double* H, const double* zb, const double* zsl, double* f_ice,
                                   double* H_grnd, double* z_srf, double* f_grnd, double rsi, double ris) {
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        double fi = (H[c] > 0.0) ? 1.0 : 0.0;
        f_ice[c] = fi;
        double d = zsl[c] - zb[c];
        double hg = (d > 0.0) ? H[c] - rsi * d : H[c] + (zb[c] - zsl[c]);
        H_grnd[c] = hg;
        double He = (fi < 1.0) ? 0.0 : H[c];
        double a = zb[c] + He, b = zsl[c] + (1.0 - ris) * He;
        z_srf[c] = (a > b) ? a : b;
        f_grnd[c] = (hg < 0.0) ? 0.0 : 1.0;
    }
}

// grounded fraction of the faces (calc_f_grnd_subgrid_linear) and the
// surface gradient (calc_gradient_acx/acy, zero_outside=.FALSE.) with the
// uniform background slope (sbx, sby) added before the limit (yelmo_tools.f90:401)
__global__ void k_inputs_faces(int nx, int ny, int bc, const double* H_grnd, const double* z_srf, double* fgx,
                               double* fgy, double* dzsdx, double* dzsdy, double dx, double grad_lim, double sbx,
                               double sby) {
    int n2 = nx * ny;
    bool px, py;
    periodic_dirs(bc, px, py);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        int i = c % nx, j = c / nx;
        // edge faces copy the neighbouring face (non-periodic directions)
        int fi = (!px && i == nx - 1) ? nx - 2 : i;
        int fj = (!py && j == ny - 1) ? ny - 2 : j;
        for (int dir = 0; dir < 2; dir++) {
            int a = dir == 0 ? fi : i, b = dir == 0 ? j : fj;
            int im1, ip1, jm1, jp1;
            nbr_bc(a, b, nx, ny, bc, im1, ip1, jm1, jp1);
            int cc = a + nx * b, cn = dir == 0 ? ip1 + nx * b : a + nx * jp1;
            double h1 = H_grnd[cc], h2 = H_grnd[cn], f;
            if (h1 > 0.0 && h2 <= 0.0) f = -h1 / (h2 - h1);
            else if (h1 <= 0.0 && h2 > 0.0) f = -h2 / (h1 - h2);
            else if (h1 <= 0.0 && h2 <= 0.0) f = 0.0;
            else f = 1.0;
            if (dir == 0) fgx[c] = f; else fgy[c] = f;
        }
        // gradients, with the edge copies of infinite / MISMIP3D / TROUGH / mask / periodic-y (x)
        // and infinite / mask / periodic-x (y)
        int gi = i, gj = j;
        if (bc == YGPU_BND_INFINITE || bc == YGPU_BND_MISMIP3D || bc == YGPU_BND_TROUGH || bc == YGPU_BND_PERIODIC_Y) {
            if (i == 0) gi = 1;
            else if (i == nx - 1) gi = nx - 2;
        }
        {
            int im1, ip1, jm1, jp1;
            nbr_bc(gi, j, nx, ny, bc, im1, ip1, jm1, jp1);
            double d = (z_srf[ip1 + nx * j] - z_srf[gi + nx * j]) / dx;
            d = d + sbx;
            if (d < -grad_lim) d = -grad_lim; else if (d > grad_lim) d = grad_lim;   // minmax
            dzsdx[c] = d;
        }
        if (bc == YGPU_BND_INFINITE || bc == YGPU_BND_PERIODIC_X) {
            if (j == 0) gj = 1;
            else if (j == ny - 1) gj = ny - 2;
        }
        {
            int im1, ip1, jm1, jp1;
            nbr_bc(i, gj, nx, ny, bc, im1, ip1, jm1, jp1);
            double d = (z_srf[i + nx * jp1] - z_srf[i + nx * gj]) / dx;
            d = d + sby;
            if (d < -grad_lim) d = -grad_lim; else if (d > grad_lim) d = grad_lim;
            dzsdy[c] = d;
        }
    }
}

// calc_ice_front (topography.f90:724-818) in gather form: a cell's code is set
// by itself (ice front) or, if ice free, by any ice-front neighbour.
__device__ int front_code(int i, int j, int nx, int ny, int bc, const double* f_ice, const double* f_grnd,
                          const double* zb, const double* zsl) {
    int c = i + nx * j;
    int im1, ip1, jm1, jp1;
    nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
    int nb[4] = {im1 + nx * j, ip1 + nx * j, i + nx * jm1, i + nx * jp1};
    int nfree = 0;
    for (int q = 0; q < 4; q++) nfree += (f_ice[nb[q]] < 1.0);
    if (f_ice[c] == 1.0 && nfree > 0) {
        if (f_grnd[c] > 0.0 && zsl[c] <= zb[c]) return MF_GRND;
        if (f_grnd[c] > 0.0) return MF_MARINE;
        return MF_FLOAT;
    }
    return MF_NONE;
}

__global__ void k_ice_front(int nx, int ny, int bc, const double* f_ice, const double* f_grnd, const double* zb,
                            const double* zsl, int* mf) {
    int n2 = nx * ny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        int i = c % nx, j = c / nx;
        int code = front_code(i, j, nx, ny, bc, f_ice, f_grnd, zb, zsl);
        if (code == MF_NONE && f_ice[c] < 1.0) {
            // an ice-free cell next to an ice front (any direction, with the
            // neighbour relation of that front cell)
            int hit = 0;
            int im1, ip1, jm1, jp1;
            nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
            int cand[4][2] = {{im1, j}, {ip1, j}, {i, jm1}, {i, jp1}};
            for (int q = 0; q < 4 && !hit; q++) {
                int a = cand[q][0], b = cand[q][1];
                if (front_code(a, b, nx, ny, bc, f_ice, f_grnd, zb, zsl) == MF_NONE) continue;
                int am1, ap1, bm1, bp1;
                nbr_bc(a, b, nx, ny, bc, am1, ap1, bm1, bp1);
                if ((am1 == i && b == j) || (ap1 == i && b == j) || (a == i && bm1 == j) || (a == i && bp1 == j)) hit = 1;
            }
            if (hit) code = (zb[c] < zsl[c]) ? MF_ICE_FREE : MF_ICE_FREE_LAND;
        }
        mf[c] = code;
    }
}

// calc_driving_stress (velocity_general.f90:1118-1205) and
// calc_lateral_bc_stress_2D (:1453-1609)
__global__ void k_stresses(int nx, int ny, int bc, const double* H, const double* f_ice, const double* dzsdx,
                           const double* dzsdy, const double* z_srf, const double* zsl, const int* mf, double* tdx,
                           double* tdy, double* tlx, double* tly, double rho_ice, double rho_sw, double g,
                           double taud_lim) {
    int n2 = nx * ny;
    double rhog = rho_ice * g;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        for (int dir = 0; dir < 2; dir++) {
            int cn = dir == 0 ? ip1 + nx * j : i + nx * jp1;
            double Hm;
            if (f_ice[c] == 1.0 && f_ice[cn] < 1.0) Hm = 0.5 * (H[c] + 0.0);
            else if (f_ice[c] < 1.0 && f_ice[cn] == 1.0) Hm = 0.5 * (0.0 + H[cn]);
            else Hm = 0.5 * (H[c] + H[cn]);
            double t = rhog * Hm * (dir == 0 ? dzsdx[c] : dzsdy[c]);
            if (t > taud_lim) t = taud_lim;
            if (t < -taud_lim) t = -taud_lim;
            if (dir == 0) tdx[c] = t; else tdy[c] = t;
            double tl = 0.0;
            if ((mf[c] > 0 && mf[cn] < 0) || (mf[c] < 0 && mf[cn] > 0)) {
                int ci = (mf[c] < 0) ? cn : c;
                double Hn = H[ci], zs = z_srf[ci], zl = zsl[ci];
                if (mf[c] == MF_ICE_FREE_LAND || mf[cn] == MF_ICE_FREE_LAND) zl = zs - Hn;
                double r = (zs - zl) / Hn;
                double fs = 1.0 - (r < 1.0 ? r : 1.0);
                double Ho = Hn * fs;
                tl = 0.5 * rho_ice * g * (Hn * Hn) - 0.5 * rho_sw * g * (Ho * Ho);
            }
            if (dir == 0) tlx[c] = tl; else tly[c] = tl;
        }
    }
}

// front_face_mask, solver_ssa_ac.f90:945-996
__device__ int front_face_mask(int a, int b, int lat) {
    int ice, fre;
    if (a > 0 && b < 0) { ice = a; fre = b; }
    else if (a < 0 && b > 0) { ice = b; fre = a; }
    else return -1;
    if (fre == MF_ICE_FREE_LAND) {
        if (ice == MF_FLOAT) return 0;
        ice = MF_GRND;
    }
    switch (lat) {
        case YGPU_LATBC_NONE: return 4;
        case YGPU_LATBC_FLOATING: return (ice == MF_FLOAT) ? 3 : 4;
        case YGPU_LATBC_MARINE: return (ice == MF_FLOAT || ice == MF_MARINE) ? 3 : 4;
        case YGPU_LATBC_ALL: return 3;
        default: return -1;
    }
}

// set_ssa_masks, solver_ssa_ac.f90:851-943
__global__ void k_ssa_masks(int nx, int ny, int bc, int lat, const int* mf, const double* f_ice, const double* f_grnd,
                            int* mx, int* my) {
    int n2 = nx * ny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        int cx = ip1 + nx * j, cy = i + nx * jp1;
        int m = 0;
        if (f_ice[c] == 1.0 || f_ice[cx] == 1.0) m = (f_grnd[c] > 0.0 || f_grnd[cx] > 0.0) ? 1 : 2;
        int ml = front_face_mask(mf[c], mf[cx], lat);
        if (ml >= 0) m = ml;
        mx[c] = m;
        m = 0;
        if (f_ice[c] == 1.0 || f_ice[cy] == 1.0) m = (f_grnd[c] > 0.0 || f_grnd[cy] > 0.0) ? 1 : 2;
        ml = front_face_mask(mf[c], mf[cy], lat);
        if (ml >= 0) m = ml;
        my[c] = m;
    }
}

static int grid_for(int n) {
    int b = (n + 255) / 256;
    return b < 1 ? 1 : (b > 4096 ? 4096 : b);
}

// device-pointer versions (stream-ordered)
int ygpu_dyn_inputs_device(cudaStream_t s, const double* H, const double* zb, const double* zsl, double* f_ice,
                           double* H_grnd, double* z_srf, double* f_grnd, double* fgx, double* fgy, int* mf,
                           double* dzsdx, double* dzsdy, double* tdx, double* tdy, double* tlx, double* tly,
                           double dx, double grad_lim, double taud_lim, double rho_ice, double rho_sw, double g,
                           int bc, int nx, int ny, double slope_bg_x, double slope_bg_y) {
    int n2 = nx * ny, gb = grid_for(n2);
    k_inputs_pointwise<<<gb, 256, 0, s>>>(n2, H, zb, zsl, f_ice, H_grnd, z_srf, f_grnd, rho_sw / rho_ice,
                                          rho_ice / rho_sw);
    k_inputs_faces<<<gb, 256, 0, s>>>(nx, ny, bc, H_grnd, z_srf, fgx, fgy, dzsdx, dzsdy, dx, grad_lim,
                                           slope_bg_x, slope_bg_y);
    k_ice_front<<<gb, 256, 0, s>>>(nx, ny, bc, f_ice, f_grnd, zb, zsl, mf);
    k_stresses<<<gb, 256, 0, s>>>(nx, ny, bc, H, f_ice, dzsdx, dzsdy, z_srf, zsl, mf, tdx, tdy, tlx, tly, rho_ice,
                                  rho_sw, g, taud_lim);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("input kernels: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(4);
    return YGPU_OK;
}

int ygpu_ssa_masks_device(cudaStream_t s, int* mx, int* my, const int* mf, const double* f_ice, const double* f_grnd,
                          int lat, int bc, int nx, int ny) {
    k_ssa_masks<<<grid_for(nx * ny), 256, 0, s>>>(nx, ny, bc, lat, mf, f_ice, f_grnd, mx, my);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("mask kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

// ---------------------------------------------------------------------------
// Post-solve diagnostics of calc_ydyn (yelmo_dynamics.f90:304-336, :642-644)
// ---------------------------------------------------------------------------
#define YG_TOL_UNDERFLOW 1e-15

// integrate_trapezoid1D_pt (yelmo_tools.f90:1092-1122) of the column of cell c
__device__ double trapz_column(const double* v, const double* zeta, int c, int n2, int nz) {
    double s = 0.0;
    for (int k = 1; k < nz; k++) {
        const double mid = 0.5 * (v[(size_t)k * n2 + c] + v[(size_t)(k - 1) * n2 + c]);
        s = s + mid * (zeta[k] - zeta[k - 1]);
    }
    return s;
}

// is_gl_face of calc_grounding_line_flux (velocity_general.f90:1873-1882)
__device__ bool gl_face(double fg0, double fg1, double fi0, double fi1) {
    return (fg0 > 0.0 && fg1 == 0.0 && fi1 > 0.0) || (fg1 > 0.0 && fg0 == 0.0 && fi0 > 0.0);
}

// depth averages of the shear velocity, ice flux (calc_ice_flux,
// velocity_general.f90:1752-1823) and grounding-line flux (:1825-1886)
__global__ void k_diag_faces(ygpu_dyn_diag D, int bc) {
    const int nx = D.nx, ny = D.ny, n2 = nx * ny;
    bool px, py;
    periodic_dirs(bc, px, py);
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        if (D.ux_i) {
            D.ux_i_bar[c] = trapz_column(D.ux_i, D.zeta_aa, c, n2, D.nz);
            D.uy_i_bar[c] = trapz_column(D.uy_i, D.zeta_aa, c, n2, D.nz);
        }
        const int cx = ip1 + nx * j, cy = i + nx * jp1;
        double qx = 0.0, qy = 0.0;
        if (i < nx - 1 || px) {
            const double area = (D.ux_bar[c] >= 0.0) ? D.H_ice[c] * D.dy : D.H_ice[cx] * D.dy;
            qx = area * D.ux_bar[c];
        }
        if (j < ny - 1 || py) {
            const double area = (D.uy_bar[c] >= 0.0) ? D.H_ice[c] * D.dx : D.H_ice[cy] * D.dx;
            qy = area * D.uy_bar[c];
        }
        D.qq_acx[c] = qx;
        D.qq_acy[c] = qy;
        D.qq_gl_acx[c] = gl_face(D.f_grnd[c], D.f_grnd[cx], D.f_ice[c], D.f_ice[cx]) ? qx : 0.0;
        D.qq_gl_acy[c] = gl_face(D.f_grnd[c], D.f_grnd[cy], D.f_ice[c], D.f_ice[cy]) ? qy : 0.0;
    }
}

// calc_magnitude_from_staggered (yelmo_tools.f90:287-339) at cell (i, j)
__device__ double mag_staggered(const double* u, const double* v, const double* f_ice, int c, int cxm, int cym) {
    double unow = 0.0, vnow = 0.0;
    if (f_ice[c] != 1.0) return 0.0;      // sqrt(0): the ice-free value, without the FP64 square root
    {
        unow = 0.5 * (u[cxm] + u[c]);
        vnow = 0.5 * (v[cym] + v[c]);
        if (fabs(unow) < YG_TOL_UNDERFLOW) unow = 0.0;
        if (fabs(vnow) < YG_TOL_UNDERFLOW) vnow = 0.0;
    }
    double m = sqrt(unow * unow + vnow * vnow);
    if (fabs(m) < YG_TOL_UNDERFLOW) m = 0.0;
    return m;
}

// magnitudes, surface fields and f_vbvs (calc_vel_ratio, velocity_general.f90:1888-1905)
__global__ void k_diag_cells(ygpu_dyn_diag D, int bc) {
    const int nx = D.nx, ny = D.ny, n2 = nx * ny, nz = D.nz;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        const int cxm = im1 + nx * j, cym = i + nx * jm1;
        D.qq[c] = mag_staggered(D.qq_acx, D.qq_acy, D.f_ice, c, cxm, cym);
        D.taub[c] = mag_staggered(D.taub_acx, D.taub_acy, D.f_ice, c, cxm, cym);
        D.taud[c] = mag_staggered(D.taud_acx, D.taud_acy, D.f_ice, c, cxm, cym);
        const double ub = mag_staggered(D.ux_b, D.uy_b, D.f_ice, c, cxm, cym);
        D.uxy_b[c] = ub;
        if (D.uxy_i_bar && D.ux_i_bar) D.uxy_i_bar[c] = mag_staggered(D.ux_i_bar, D.uy_i_bar, D.f_ice, c, cxm, cym);
        D.uxy_bar[c] = mag_staggered(D.ux_bar, D.uy_bar, D.f_ice, c, cxm, cym);
        if (D.ux) {
            double us = 0.0;
            for (int k = 0; k < nz; k++) {
                const size_t o = (size_t)k * n2;
                us = mag_staggered(D.ux + o, D.uy + o, D.f_ice, c, cxm, cym);
                D.uxy[o + c] = us;
            }
            const size_t top = (size_t)(nz - 1) * n2;
            D.ux_s[c] = D.ux[top + c];
            D.uy_s[c] = D.uy[top + c];
            D.uxy_s[c] = us;
            D.f_vbvs[c] = (us > 0.0) ? fmin(1.0, ub / us) : 1.0;
        }
    }
}

int ygpu_dyn_diagnostics_device(cudaStream_t s, const ygpu_dyn_diag& D, int bc) {
    const int gb = grid_for(D.nx * D.ny);
    k_diag_faces<<<gb, 256, 0, s>>>(D, bc);
    k_diag_cells<<<gb, 256, 0, s>>>(D, bc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("diagnostic kernels: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(2);
    return YGPU_OK;
}

// ---------------------------------------------------------------------------
// Column gradients and the velocity Jacobian of calc_ydyn
// (src/yelmo_dynamics.f90:243-296)
// ---------------------------------------------------------------------------

// calc_gradient_column_ac (yelmo_tools.f90:479-571): the face keeps its
// gradient between two ice-covered cells and at a margin to ice-free land; at a
// face to ice-free ocean it takes the ice-side neighbour face if that face lies
// between two ice-covered cells; otherwise zero.
__global__ void k_gradient_column(int nx, int ny, int bc, const double* __restrict__ gx,
                                  const double* __restrict__ gy, const double* __restrict__ f_ice,
                                  const int* __restrict__ ocn, double* __restrict__ gx_c, double* __restrict__ gy_c) {
    const int n2 = nx * ny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        {
            const int c1 = ip1 + nx * j;
            const bool ice0 = f_ice[c] == 1.0, ice1 = f_ice[c1] == 1.0;
            double v = 0.0;
            if (ice0 && ice1) {
                v = gx[c];
            } else if ((ice0 && !ocn[c1]) || (ice1 && !ocn[c])) {
                v = gx[c];
            } else if (ice0) {
                if (im1 != i && f_ice[im1 + nx * j] == 1.0) v = gx[im1 + nx * j];
            } else if (ice1) {
                int am1, ap1, bm1, bp1;
                nbr_bc(ip1, j, nx, ny, bc, am1, ap1, bm1, bp1);
                if (ap1 != ip1 && f_ice[ap1 + nx * j] == 1.0) v = gx[c1];
            }
            gx_c[c] = v;
        }
        {
            const int c1 = i + nx * jp1;
            const bool ice0 = f_ice[c] == 1.0, ice1 = f_ice[c1] == 1.0;
            double v = 0.0;
            if (ice0 && ice1) {
                v = gy[c];
            } else if ((ice0 && !ocn[c1]) || (ice1 && !ocn[c])) {
                v = gy[c];
            } else if (ice0) {
                if (jm1 != j && f_ice[i + nx * jm1] == 1.0) v = gy[i + nx * jm1];
            } else if (ice1) {
                int am1, ap1, bm1, bp1;
                nbr_bc(i, jp1, nx, ny, bc, am1, ap1, bm1, bp1);
                if (bp1 != jp1 && f_ice[i + nx * bp1] == 1.0) v = gy[c1];
            }
            gy_c[c] = v;
        }
    }
}

// calc_active_faces (deformation.f90:1316-1344) of the x face right of (a, b)
// and of the y face above it
YG_DEV bool jac_act_x(const double* f, int a, int b, int nx, int ny, int bc) {
    int am1, ap1, bm1, bp1;
    nbr_bc(a, b, nx, ny, bc, am1, ap1, bm1, bp1);
    return f[a + nx * b] == 1.0 || f[ap1 + nx * b] == 1.0;
}
YG_DEV bool jac_act_y(const double* f, int a, int b, int nx, int ny, int bc) {
    int am1, ap1, bm1, bp1;
    nbr_bc(a, b, nx, ny, bc, am1, ap1, bm1, bp1);
    return f[a + nx * b] == 1.0 || f[a + nx * bp1] == 1.0;
}

// mean4_active (deformation.f90:1370-1391); the count's reciprocal from a table
YG_DEV double jac_mean4(double v1, double v2, double v3, double v4, bool a1, bool a2, bool a3, bool a4) {
    const int n = (int)a1 + (int)a2 + (int)a3 + (int)a4;
    double s = (a1 ? v1 : 0.0) + (a2 ? v2 : 0.0);
    s = s + (a3 ? v3 : 0.0);
    s = s + (a4 ? v4 : 0.0);
    const double r = n == 4 ? 0.25 : n == 2 ? 0.5 : n == 1 ? 1.0 : n == 3 ? (1.0 / 3.0) : 0.0;
    return s * r;
}

// FP64 on this GPU issues at 2 FMA per clock per SM, so the Jacobian keeps every
// division out of its layer loops. The three-point unequal-spacing derivative of
// the reference (Singh and Bhadauria; deformation.f90:508-540, :805-836) is
// rewritten in difference form,
//     du/dz (k) = (a_k (u[p] - u[p-1]) + b_k (u[p+1] - u[p])) / H,  p = clamp(k, 1, nz-2),
// with the layer weights a_k, b_k of the zeta spacing (the same polynomial, the
// thickness factored out). The top layer of uz takes the first-order difference
// (a = 0). The weights are computed once per block into shared memory.
YG_DEV void jac_layer_weights(const double* z, int nz, int k, bool top3, double& a, double& b) {
    if (k == 0) {
        const double d1 = z[1] - z[0], d2 = z[2] - z[1];
        a = (2.0 * d1 + d2) / (d1 * (d1 + d2));
        b = -d1 / (d2 * (d1 + d2));
    } else if (k < nz - 1) {
        const double d1 = z[k] - z[k - 1], d2 = z[k + 1] - z[k];
        a = d2 / (d1 * (d1 + d2));
        b = d1 / (d2 * (d1 + d2));
    } else if (top3) {
        const double d1 = z[k - 1] - z[k - 2], d2 = z[k] - z[k - 1];
        a = -d2 / (d1 * (d1 + d2));
        b = (d1 + 2.0 * d2) / (d2 * (d1 + d2));
    } else {
        a = 0.0;
        b = 1.0 / (z[k] - z[k - 1]);
    }
}

// Running pair of layer differences (u[p] - u[p-1], u[p+1] - u[p]) of one column
struct JacWindow {
    const double* u;
    size_t c, n2;
    int p, nz;
    double up, dA, dB;
    YG_DEV void init(const double* u_, size_t c_, size_t n2_, int nz_) {
        u = u_; c = c_; n2 = n2_; nz = nz_; p = 1;
        const double u0 = __ldg(u + c), u1 = __ldg(u + n2 + c);
        up = __ldg(u + 2 * n2 + c);
        dA = u1 - u0;
        dB = up - u1;
    }
    // the derivative at layer k (k ascending), times rH = 1/H
    YG_DEV double at(int k, double a, double b, double rH) {
        if (k > p && k < nz - 1) {
            p = k;
            const double un = __ldg(u + (size_t)(k + 1) * n2 + c);
            dA = dB;
            dB = un - up;
            up = un;
        }
        return fma(b, dB, a * dA) * rH;
    }
};

// A horizontal derivative as s1 (u[a] - u[b]) + s2 (u[cc] - u[d]) over the
// offsets of one layer, chosen once per column so that the layer loop carries
// no branch. Margin stencils (deformation.f90:590-637, :866-929): mode 0
// centred, 1 three-point backward, 2 two-point backward, 3 three-point forward,
// 4 two-point forward, 5 zero; r1 = 1/h, r2 = 1/(2h). The three-point forms
// are the reference's (u[-2] - 4 u[-1] + 3 u[0]) / 2h regrouped as
// 3/2h (u[0] - u[-1]) - 1/2h (u[-1] - u[-2]) (and mirrored).
struct JacTap {
    int a, b, cc, d;
    double s1, s2;
};

YG_DEV JacTap jac_tap_margin(int mode, int m2, int m1, int c0, int p1, int p2, double r1, double r2) {
    switch (mode) {
        case 1: return {c0, m1, m1, m2, 3.0 * r2, -r2};
        case 2: return {c0, m1, c0, c0, r1, 0.0};
        case 3: return {p1, c0, p2, p1, 3.0 * r2, -r2};
        case 4: return {p1, c0, c0, c0, r1, 0.0};
        case 5: return {c0, c0, c0, c0, 0.0, 0.0};
        default: return {p1, m1, c0, c0, r2, 0.0};
    }
}

// deriv_active (deformation.f90:1346-1368) as a one-difference tap
YG_DEV JacTap jac_tap_active(int m, int c0, int p, bool am, bool ap, double r1, double r2) {
    if (am && ap) return {p, m, c0, c0, r2, 0.0};
    if (ap) return {p, c0, c0, c0, r1, 0.0};
    if (am) return {c0, m, c0, c0, r1, 0.0};
    return {c0, c0, c0, c0, 0.0, 0.0};
}

YG_DEV double jac_tap2(const JacTap& t, const double* __restrict__ u) {
    return fma(t.s2, __ldg(u + t.cc) - __ldg(u + t.d), t.s1 * (__ldg(u + t.a) - __ldg(u + t.b)));
}
YG_DEV double jac_tap1(const JacTap& t, const double* __restrict__ u) {
    return t.s1 * (__ldg(u + t.a) - __ldg(u + t.b));
}

struct JacConst {
    double rdx, r2dx, rdy, r2dy;
    const double *wa_aa, *wb_aa, *z_aa, *wa_ac, *wb_ac, *z_ac;   // shared memory
};

// calc_jacobian_vel_3D_uxyterms (deformation.f90:397-716) for the column at (i, j)
YG_DEV void jac_uxy_column(const ygpu_jvel& J, const JacConst& K, int bc, int i, int j, int im1, int ip1, int jm1,
                           int jp1) {
    const int nx = J.nx, ny = J.ny, nz = J.nz_aa;
    const size_t n2 = (size_t)nx * ny, c = (size_t)i + (size_t)nx * j;
    const double* __restrict__ f = J.f_ice;
    const double* __restrict__ H = J.H_ice;
    const size_t cxp = ip1 + (size_t)nx * j, cxm = im1 + (size_t)nx * j;
    const size_t cyp = i + (size_t)nx * jp1, cym = i + (size_t)nx * jm1;
    const bool ice = f[c] == 1.0, ice_xp = f[cxp] == 1.0, ice_yp = f[cyp] == 1.0;
    const bool less = f[c] < 1.0, less_xp = f[cxp] < 1.0, less_yp = f[cyp] < 1.0;
    // face thicknesses (:473-487)
    double Hx, Hy;
    if (ice && less_xp) Hx = H[c];
    else if (less && ice_xp) Hx = H[cxp];
    else Hx = 0.5 * (H[c] + H[cxp]);
    if (ice && less_yp) Hy = H[c];
    else if (less && ice_yp) Hy = H[cyp];
    else Hy = 0.5 * (H[c] + H[cyp]);
    const double rHx = Hx > 0.0 ? 1.0 / Hx : 0.0, rHy = Hy > 0.0 ? 1.0 / Hy : 0.0;
    // margin stencils of dxx and dyy (:590-637)
    int mx = 0, my = 0;
    if (ice && less_xp) mx = (im1 > 0 && f[cxm] == 1.0) ? 1 : 2;
    else if (less && ice_xp) mx = (ip1 < nx - 1 && f[cxp + 1] == 1.0) ? 3 : 4;
    if (ice && less_yp) my = (jm1 > 0 && f[cym] == 1.0) ? 1 : 2;
    else if (less && ice_yp) my = (jp1 < ny - 1 && f[cyp + nx] == 1.0) ? 3 : 4;
    // faces with a velocity solution and the cross gradients over them (:654-666)
    const bool ax_jm1 = jac_act_x(f, i, jm1, nx, ny, bc), ax_jp1 = jac_act_x(f, i, jp1, nx, ny, bc);
    const bool ax_0 = jac_act_x(f, i, j, nx, ny, bc), ax_im1 = jac_act_x(f, im1, j, nx, ny, bc);
    const bool ax_im1_jp1 = jac_act_x(f, im1, jp1, nx, ny, bc);
    const bool ay_im1 = jac_act_y(f, im1, j, nx, ny, bc), ay_ip1 = jac_act_y(f, ip1, j, nx, ny, bc);
    const bool ay_0 = jac_act_y(f, i, j, nx, ny, bc), ay_jm1 = jac_act_y(f, i, jm1, nx, ny, bc);
    const bool ay_ip1_jm1 = jac_act_y(f, ip1, jm1, nx, ny, bc);
    const double* bx = J.dzbdx;
    const double* by = J.dzbdy;
    const double* sx = J.dzsdx;
    const double* sy = J.dzsdy;
    const size_t cxm_yp = im1 + (size_t)nx * jp1, cxp_ym = ip1 + (size_t)nx * jm1;
    const double bx_acy = jac_mean4(bx[c], bx[cyp], bx[cxm], bx[cxm_yp], ax_0, ax_jp1, ax_im1, ax_im1_jp1);
    const double sx_acy = jac_mean4(sx[c], sx[cyp], sx[cxm], sx[cxm_yp], ax_0, ax_jp1, ax_im1, ax_im1_jp1);
    const double by_acx = jac_mean4(by[c], by[cxp], by[cym], by[cxp_ym], ay_0, ay_ip1, ay_jm1, ay_ip1_jm1);
    const double sy_acx = jac_mean4(sy[c], sy[cxp], sy[cym], sy[cxp_ym], ay_0, ay_ip1, ay_jm1, ay_ip1_jm1);
    // sigma-transform factors (:639-675): c(zeta) = -((1-zeta) b + zeta s) = -(b + zeta (s - b))
    const double bxc = bx[c], byc = by[c];
    const double gxc = sx[c] - bxc, gyc = sy[c] - byc, gx_acy = sx_acy - bx_acy, gy_acx = sy_acx - by_acx;
    const double* __restrict__ ux = J.ux;
    const double* __restrict__ uy = J.uy;
    // horizontal stencils of this column (offsets within a layer)
    const int ic = (int)c, ixm = (int)cxm, ixp = (int)cxp, iym = (int)cym, iyp = (int)cyp;
    const JacTap txx = jac_tap_margin(mx, mx == 1 ? ixm - 1 : ic, ixm, ic, ixp, mx == 3 ? ixp + 1 : ic, K.rdx, K.r2dx);
    const JacTap tyy = jac_tap_margin(my, my == 1 ? iym - nx : ic, iym, ic, iyp, my == 3 ? iyp + nx : ic, K.rdy, K.r2dy);
    const JacTap txy = jac_tap_active(iym, ic, iyp, ax_jm1, ax_jp1, K.rdy, K.r2dy);
    const JacTap tyx = jac_tap_active(ixm, ic, ixp, ay_im1, ay_ip1, K.rdx, K.r2dx);
    JacWindow wx, wy;
    wx.init(ux, c, n2, nz);
    wy.init(uy, c, n2, nz);
    for (int k = 0; k < nz; k++) {
        const size_t o = (size_t)k * n2;
        const double wa = K.wa_aa[k], wb = K.wb_aa[k], zk = K.z_aa[k];
        const double dxz = (Hx > 0.0) ? wx.at(k, wa, wb, rHx) : 0.0;
        const double dyz = (Hy > 0.0) ? wy.at(k, wa, wb, rHy) : 0.0;
        const double* uxk = ux + o;
        const double* uyk = uy + o;
        double dxx = jac_tap2(txx, uxk);
        double dyy = jac_tap2(tyy, uyk);
        double dxy = jac_tap1(txy, uxk);
        double dyx = jac_tap1(tyx, uyk);
        dxx = fma(-fma(zk, gxc, bxc), dxz, dxx);
        dxy = fma(-fma(zk, gy_acx, by_acx), dxz, dxy);
        dyx = fma(-fma(zk, gx_acy, bx_acy), dyz, dyx);
        dyy = fma(-fma(zk, gyc, byc), dyz, dyy);
        J.dxx[o + c] = dxx;
        J.dxy[o + c] = dxy;
        J.dxz[o + c] = dxz;
        J.dyx[o + c] = dyx;
        J.dyy[o + c] = dyy;
        J.dyz[o + c] = dyz;
    }
}

// calc_jacobian_vel_3D_uzterms (deformation.f90:718-961) for the column at (i, j)
YG_DEV void jac_uz_column(const ygpu_jvel& J, const JacConst& K, int i, int j, int im1, int ip1, int jm1, int jp1) {
    const int nx = J.nx, ny = J.ny, nz = J.nz_ac;
    const size_t n2 = (size_t)nx * ny, c = (size_t)i + (size_t)nx * j;
    const double* __restrict__ f = J.f_ice;
    if (!(f[c] == 1.0)) {
        for (int k = 0; k < nz; k++) {
            const size_t o = (size_t)k * n2 + c;
            J.dzx[o] = 0.0;
            J.dzy[o] = 0.0;
            J.dzz[o] = 0.0;
        }
        return;
    }
    const size_t cxp = ip1 + (size_t)nx * j, cxm = im1 + (size_t)nx * j;
    const size_t cyp = i + (size_t)nx * jp1, cym = i + (size_t)nx * jm1;
    const bool exp_ = f[cxp] == 1.0, exm = f[cxm] == 1.0, eyp = f[cyp] == 1.0, eym = f[cym] == 1.0;
    const bool lxp = f[cxp] < 1.0, lxm = f[cxm] < 1.0, lyp = f[cyp] < 1.0, lym = f[cym] < 1.0;
    int mx = 0, my = 0;
    if (lxp && lxm) mx = 5;
    else if (lxp && exm) mx = (im1 > 0 && f[cxm - 1] == 1.0) ? 1 : 2;
    else if (exp_ && lxm) mx = (ip1 < nx - 1 && f[cxp + 1] == 1.0) ? 3 : 4;
    if (lyp && lym) my = 5;
    else if (lyp && eym) my = (jm1 > 0 && f[cym - nx] == 1.0) ? 1 : 2;
    else if (eyp && lym) my = (jp1 < ny - 1 && f[cyp + nx] == 1.0) ? 3 : 4;
    const double rH = 1.0 / J.H_ice[c];
    // correction factors on the cell (:935-944)
    const double bxa = 0.5 * (J.dzbdx[c] + J.dzbdx[cxm]), bya = 0.5 * (J.dzbdy[c] + J.dzbdy[cym]);
    const double gxa = 0.5 * (J.dzsdx[c] + J.dzsdx[cxm]) - bxa, gya = 0.5 * (J.dzsdy[c] + J.dzsdy[cym]) - bya;
    const int ic = (int)c, ixm = (int)cxm, ixp = (int)cxp, iym = (int)cym, iyp = (int)cyp;
    const JacTap tzx = jac_tap_margin(mx, mx == 1 ? ixm - 1 : ic, ixm, ic, ixp, mx == 3 ? ixp + 1 : ic, K.rdx, K.r2dx);
    const JacTap tzy = jac_tap_margin(my, my == 1 ? iym - nx : ic, iym, ic, iyp, my == 3 ? iyp + nx : ic, K.rdy, K.r2dy);
    const double* __restrict__ uz = J.uz;
    JacWindow wz;
    wz.init(uz, c, n2, nz);
    for (int k = 0; k < nz; k++) {
        const size_t o = (size_t)k * n2;
        const double* uzk = uz + o;
        const double dzz = wz.at(k, K.wa_ac[k], K.wb_ac[k], rH);
        const double zk = K.z_ac[k];
        const double dzx = fma(-fma(zk, gxa, bxa), dzz, jac_tap2(tzx, uzk));
        const double dzy = fma(-fma(zk, gya, bya), dzz, jac_tap2(tzy, uzk));
        J.dzx[o + c] = dzx;
        J.dzy[o + c] = dzy;
        J.dzz[o + c] = dzz;
    }
}

// One thread per column: the ux/uy terms, then the uz terms (or the zeroing of
// dzx, dzy, dzz that the ux/uy routine starts with). Dynamic shared memory:
// the layer weights and levels, 3 (nz_aa + nz_ac) doubles.
__global__ void __launch_bounds__(256) k_jacobian(ygpu_jvel J, int bc, int terms) {
    extern __shared__ double jac_sh[];
    const int nza = (terms & YGPU_JAC_UXY) ? J.nz_aa : 0, nzc = (terms & YGPU_JAC_UZ) ? J.nz_ac : 0;
    JacConst K;
    double* wa_aa = jac_sh;
    double* wb_aa = wa_aa + nza;
    double* z_aa = wb_aa + nza;
    double* wa_ac = z_aa + nza;
    double* wb_ac = wa_ac + nzc;
    double* z_ac = wb_ac + nzc;
    for (int k = threadIdx.x; k < nza; k += blockDim.x) {
        jac_layer_weights(J.zeta_aa, nza, k, true, wa_aa[k], wb_aa[k]);
        z_aa[k] = J.zeta_aa[k];
    }
    for (int k = threadIdx.x; k < nzc; k += blockDim.x) {
        jac_layer_weights(J.zeta_ac, nzc, k, false, wa_ac[k], wb_ac[k]);
        z_ac[k] = J.zeta_ac[k];
    }
    __syncthreads();
    K.wa_aa = wa_aa; K.wb_aa = wb_aa; K.z_aa = z_aa;
    K.wa_ac = wa_ac; K.wb_ac = wb_ac; K.z_ac = z_ac;
    K.rdx = 1.0 / J.dx; K.r2dx = 1.0 / (2.0 * J.dx);
    K.rdy = 1.0 / J.dy; K.r2dy = 1.0 / (2.0 * J.dy);
    const int nx = J.nx, ny = J.ny, n2 = nx * ny;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n2; c += gridDim.x * blockDim.x) {
        const int i = c % nx, j = c / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        if (terms & YGPU_JAC_UXY) jac_uxy_column(J, K, bc, i, j, im1, ip1, jm1, jp1);
        if (terms & YGPU_JAC_UZ) {
            jac_uz_column(J, K, i, j, im1, ip1, jm1, jp1);
        } else if (J.dzx) {
            for (int k = 0; k < J.nz_ac; k++) {
                const size_t o = (size_t)k * n2 + c;
                J.dzx[o] = 0.0;
                J.dzy[o] = 0.0;
                J.dzz[o] = 0.0;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Vertical velocity (calc_uz_3D_aa / calc_uz_3D_flux, velocity_general.f90:683-1116)
// ---------------------------------------------------------------------------

// |v| < 1e-15 -> 0, evaluated on the integer pipe: the magnitude bits of a
// double order like its absolute value (NaN and inf compare above any finite
// bound), so the test is the same as fabs(v) < 1e-15 without an FP64 compare.
YG_DEV double flush_tiny(double v) {
    const unsigned long long mag = (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull;
    return mag < (unsigned long long)__double_as_longlong(YG_TOL_UNDERFLOW) ? 0.0 : v;
}

// Horizontal velocity at level kc of the interfaces, times 4, from the face sums
// of the layers sa(k) = u[im1] + u[i]: the base and top layers at the ends, the
// two adjacent layers between (velocity_general.f90:850-866, where the level
// value is their mean).
YG_DEV double uz_level_sum4(int kc, int nzc, double sa_k, double sa_km1) {
    if (kc == 0) return sa_k + sa_k;
    if (kc == nzc - 1) return sa_km1 + sa_km1;
    return sa_k + sa_km1;
}

// One thread per column. Shared memory: zeta_ac, its spacing dzc[kc] =
// zeta_ac[kc] - zeta_ac[kc-1] and, for YGPU_UZ_AA, half the reciprocal spacing
// of the zeta_aa pair of the vertical derivative at each level (3 nz_ac doubles).
// FP64 issues at 2 FMA per clock per SM on this GPU: the level loops carry face
// sums instead of means, the 1/2 and 1/4 of the means sit in per-column
// constants (exact power-of-two scalings), and the coordinate terms are FMAs.
__global__ void __launch_bounds__(256) k_uz3d(ygpu_uz3d U, int bc, int method) {
    extern __shared__ double uz_sh[];
    const int nza = U.nz_aa, nzc = U.nz_ac;
    double* zc = uz_sh;
    double* dzc = zc + nzc;
    double* hrdz = dzc + nzc;
    for (int k = threadIdx.x; k < nzc; k += blockDim.x) {
        zc[k] = U.zeta_ac[k];
        dzc[k] = k > 0 ? U.zeta_ac[k] - U.zeta_ac[k - 1] : 0.0;
        int hi = k, lo = k - 2;                        // centred on layer k-1
        if (k <= 1) { hi = 1; lo = 0; }
        else if (k == nzc - 1) { hi = nza - 1; lo = nza - 2; }
        hrdz[k] = 0.5 / (U.zeta_aa[hi] - U.zeta_aa[lo]);
    }
    __syncthreads();
    const double rdx = 1.0 / U.dx, rdy = 1.0 / U.dy, f_bmb = U.use_bmb ? 1.0 : 0.0;
    const int nx = U.nx, ny = U.ny;
    const size_t n2 = (size_t)nx * ny;
    const double* __restrict__ ux = U.ux;
    const double* __restrict__ uy = U.uy;
    for (int cc = blockIdx.x * blockDim.x + threadIdx.x; cc < nx * ny; cc += gridDim.x * blockDim.x) {
        const int i = cc % nx, j = cc / nx;
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        const size_t c = cc, cxm = im1 + (size_t)nx * j, cym = i + (size_t)nx * jm1;
        const double dzbdt = U.dzbdt[c], dzsdt = U.dzsdt[c];
        double top_star = 0.0;
        if (!(U.f_ice[c] == 1.0)) {
            const double u = flush_tiny(dzbdt - fmax(U.smb[c], 0.0));
            for (int kc = 0; kc < nzc; kc++) {
                U.uz[(size_t)kc * n2 + c] = u;
                U.uz_star[(size_t)kc * n2 + c] = u;
            }
            if (U.uz_srf_err) U.uz_srf_err[c] = 0.0;
            continue;
        }
        const double H = U.H_ice[c];
        const double bxa = 0.5 * (U.dzbdx[c] + U.dzbdx[cxm]), bya = 0.5 * (U.dzbdy[c] + U.dzbdy[cym]);
        const double gxa = 0.5 * (U.dzsdx[c] + U.dzsdx[cxm]) - bxa, gya = 0.5 * (U.dzsdy[c] + U.dzsdy[cym]) - bya;
        // slopes of the coordinate terms at level z: fma(z, g4, b4) = ((1-z) dzb + z dzs) / 4
        const double bx4 = 0.25 * bxa, gx4 = 0.25 * gxa, by4 = 0.25 * bya, gy4 = 0.25 * gya;
        const double gt = dzsdt - dzbdt;
        auto SA = [&](int k) { return __ldg(ux + (size_t)k * n2 + c) + __ldg(ux + (size_t)k * n2 + cxm); };
        auto SV = [&](int k) { return __ldg(uy + (size_t)k * n2 + c) + __ldg(uy + (size_t)k * n2 + cym); };
        // the coordinate terms at level kc (:867-876): c_x = -(tx/4) ((1-z) dzbdx + z dzsdx)
        // = -tx fma(z, gx4, bx4), c_y likewise, c_t = -fma(z, gt, dzbdt);
        // plus_c(v) = v + c_x + c_y + c_t, minus_c(v) = v - (c_x + c_y + c_t)
        auto plus_c = [&](double v, int kc, double tx, double ty) {
            const double z = zc[kc];
            v = v - fma(z, gt, dzbdt);
            v = fma(-tx, fma(z, gx4, bx4), v);
            return fma(-ty, fma(z, gy4, by4), v);
        };
        auto minus_c = [&](double v, int kc, double tx, double ty) {
            const double z = zc[kc];
            v = v + fma(z, gt, dzbdt);
            v = fma(tx, fma(z, gx4, bx4), v);
            return fma(ty, fma(z, gy4, by4), v);
        };
        if (method == YGPU_UZ_AA) {
            const double r4H = 4.0 / H;
            double sa_m2 = 0.0, sv_m2 = 0.0, sa_m1 = 0.0, sv_m1 = 0.0;
            double sa_0 = SA(0), sv_0 = SV(0);
            // basal value (:776-778), ux_aa = sa/2
            double uz = flush_tiny(dzbdt + f_bmb * U.bmb[c] + (0.5 * sa_0) * bxa + (0.5 * sv_0) * bya);
            for (int kc = 0; kc < nzc; kc++) {
                if (kc > 0) {
                    // window: sa_0 = layer kc (if any), sa_m1 = kc-1, sa_m2 = kc-2
                    sa_m2 = sa_m1; sv_m2 = sv_m1;
                    sa_m1 = sa_0; sv_m1 = sv_0;
                    if (kc < nza) { sa_0 = SA(kc); sv_0 = SV(kc); }
                    const int ka = kc - 1;
                    const double duxdx = (__ldg(ux + (size_t)ka * n2 + c) - __ldg(ux + (size_t)ka * n2 + cxm)) * rdx;
                    const double duydy = (__ldg(uy + (size_t)ka * n2 + c) - __ldg(uy + (size_t)ka * n2 + cym)) * rdy;
                    double dsx, dsy;                           // sa(hi) - sa(lo)
                    if (kc == 1) { dsx = sa_0 - sa_m1; dsy = sv_0 - sv_m1; }
                    else if (kc == nzc - 1) { dsx = sa_m1 - sa_m2; dsy = sv_m1 - sv_m2; }
                    else { dsx = sa_0 - sa_m2; dsy = sv_0 - sv_m2; }
                    // c_x duxdz = -(1/H) ((1-z) dzb + z dzs) (sa(hi) - sa(lo)) / (2 dzeta)
                    const double z = zc[kc];
                    const double cx = -r4H * hrdz[kc] * fma(z, gx4, bx4), cy = -r4H * hrdz[kc] * fma(z, gy4, by4);
                    const double div = fma(cx, dsx, duxdx) + fma(cy, dsy, duydy);
                    uz = flush_tiny(fma(-(H * dzc[kc]), div, uz));
                }
                // uz_star (:845-880)
                const double tx = uz_level_sum4(kc, nzc, kc < nza ? sa_0 : 0.0, sa_m1);
                const double ty = uz_level_sum4(kc, nzc, kc < nza ? sv_0 : 0.0, sv_m1);
                const double us = flush_tiny(plus_c(uz, kc, tx, ty));
                const size_t o = (size_t)kc * n2 + c;
                U.uz[o] = uz;
                U.uz_star[o] = us;
                top_star = us;
            }
        } else {
            // calc_uz_3D_flux: layer divergences with upwind face thickness (:1043-1056)
            const double* Hi = U.H_ice;
            const size_t cxp = ip1 + (size_t)nx * j, cyp = i + (size_t)nx * jp1;
            const double Hx_w = (U.ux_bar[cxm] >= 0.0) ? Hi[cxm] : Hi[c];
            const double Hx_e = (U.ux_bar[c] >= 0.0) ? Hi[c] : Hi[cxp];
            const double Hy_s = (U.uy_bar[cym] >= 0.0) ? Hi[cym] : Hi[c];
            const double Hy_n = (U.uy_bar[c] >= 0.0) ? Hi[c] : Hi[cyp];
            const double ex = Hx_e * rdx, wx = Hx_w * rdx, ny_ = Hy_n * rdy, sy = Hy_s * rdy;
            auto Dk = [&](int k) {
                const size_t o = (size_t)k * n2;
                const double fx = fma(ex, __ldg(ux + o + c), -(wx * __ldg(ux + o + cxm)));
                const double fl = fma(ny_, __ldg(uy + o + c), fma(-sy, __ldg(uy + o + cym), fx));
                return dzc[k + 1] * fl;
            };
            double q = gt;                                 // dzeta-weighted rate per layer
            if (U.mask_kin[c] == 1) {
                double tot = 0.0;
                for (int k = 0; k < nza; k++) tot += Dk(k);
                q = gt + (-U.dHidt_dyn[c] - tot);          // dHdt + D_corr
            }
            double us = f_bmb * U.bmb[c];
            double sa_m1 = 0.0, sv_m1 = 0.0, sa_0 = SA(0), sv_0 = SV(0);
            for (int kc = 0; kc < nzc; kc++) {
                if (kc > 0) {
                    us = fma(-dzc[kc], q, us) - Dk(kc - 1);
                    sa_m1 = sa_0; sv_m1 = sv_0;
                    if (kc < nza) { sa_0 = SA(kc); sv_0 = SV(kc); }
                }
                const double tx = uz_level_sum4(kc, nzc, kc < nza ? sa_0 : 0.0, sa_m1);
                const double ty = uz_level_sum4(kc, nzc, kc < nza ? sv_0 : 0.0, sv_m1);
                const size_t o = (size_t)kc * n2 + c;
                U.uz[o] = flush_tiny(minus_c(us, kc, tx, ty));
                U.uz_star[o] = flush_tiny(us);
                top_star = flush_tiny(us);
            }
        }
        if (U.uz_srf_err) U.uz_srf_err[c] = top_star + U.smb[c];
    }
}

int ygpu_uz3d_device(cudaStream_t s, const ygpu_uz3d& U, int bc, int method) {
    if (method == YGPU_UZ_NODES || method == YGPU_UZ_JAC) return ygpu_uz3d_quad_device(s, U, bc, method);
    const size_t smem = 3 * sizeof(double) * (size_t)U.nz_ac;
    k_uz3d<<<grid_for(U.nx * U.ny), 256, smem, s>>>(U, bc, method);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("vertical velocity kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

int ygpu_gradient_column_device(cudaStream_t s, double* gx_c, double* gy_c, const double* gx, const double* gy,
                                const double* f_ice, const int* mask_ocn, int bc, int nx, int ny) {
    k_gradient_column<<<grid_for(nx * ny), 256, 0, s>>>(nx, ny, bc, gx, gy, f_ice, mask_ocn, gx_c, gy_c);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("column gradient kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

int ygpu_jacobian_device(cudaStream_t s, const ygpu_jvel& J, int bc, int terms) {
    const int nza = (terms & YGPU_JAC_UXY) ? J.nz_aa : 0, nzc = (terms & YGPU_JAC_UZ) ? J.nz_ac : 0;
    const size_t smem = 3 * sizeof(double) * (size_t)(nza + nzc);
    k_jacobian<<<grid_for(J.nx * J.ny), 256, smem, s>>>(J, bc, terms);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("Jacobian kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}
