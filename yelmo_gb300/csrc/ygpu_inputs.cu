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
// surface gradient (calc_gradient_acx/acy, zero_outside=.FALSE.)
__global__ void k_inputs_faces(int nx, int ny, int bc, const double* H_grnd, const double* z_srf, double* fgx,
                               double* fgy, double* dzsdx, double* dzsdy, double dx, double grad_lim) {
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
                           int bc, int nx, int ny) {
    int n2 = nx * ny, gb = grid_for(n2);
    k_inputs_pointwise<<<gb, 256, 0, s>>>(n2, H, zb, zsl, f_ice, H_grnd, z_srf, f_grnd, rho_sw / rho_ice,
                                          rho_ice / rho_sw);
    k_inputs_faces<<<gb, 256, 0, s>>>(nx, ny, bc, H_grnd, z_srf, fgx, fgy, dzsdx, dzsdy, dx, grad_lim);
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
