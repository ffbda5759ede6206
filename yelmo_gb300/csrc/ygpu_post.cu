// ygpu_post.cu -- the routines of calc_ydyn that take fields to quadrature
// nodes, on the GPU: the vertical velocity by uz_method 2 (calc_uz_3D,
// velocity_general.f90:346-681) and 3 (calc_uz_3D_jac, :41-344, the namelist
// default), and the strain-rate tensor (calc_strain_rate_tensor_jac_quad3D,
// deformation.f90:963-1183).
//
// The quadrature restates fesm-utils' gq2D / gq3D: corner values are means of
// the active faces (acx / acy fields) or of the four cells (fields on the cell
// centres) around a cell corner, in 3D also over the two layers or ac levels
// that meet there; the Gauss-Legendre nodes at +-1/sqrt(3) interpolate them
// bilinearly (trilinearly) and the equal-weight node mean is the cell value.
// That mean equals the mean of the corners, which these kernels compute
// directly: per column, the weight of each of the six faces (or nine cells) in
// the cell value is found once, since the active faces do not change with the
// layer, and the 3D value of layer k is the 1-2-1 mean of the layers' 2D values
// (k-1, k, k+1, clamped at the base and the surface). They agree with the
// node-by-node evaluation to rounding.
//
// One thread per column, FP64.
#include <cuda_runtime.h>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

namespace {

YG_DEV double flush15(double v) { return fabs(v) < 1e-15 ? 0.0 : v; }

YG_DEV int cid(int i, int j, int nx) { return i + nx * j; }

// x face (ii, jj) carries a velocity solution: f_ice == 1 on either side
// (calc_active_faces, deformation.f90:1316-1344)
YG_DEV bool act_x(const double* f_ice, int ii, int jj, int nx, int ny, int bc) {
    int im1, ip1, jm1, jp1;
    nbr_bc(ii, jj, nx, ny, bc, im1, ip1, jm1, jp1);
    return f_ice[cid(ii, jj, nx)] == 1.0 || f_ice[cid(ip1, jj, nx)] == 1.0;
}
YG_DEV bool act_y(const double* f_ice, int ii, int jj, int nx, int ny, int bc) {
    int im1, ip1, jm1, jp1;
    nbr_bc(ii, jj, nx, ny, bc, im1, ip1, jm1, jp1);
    return f_ice[cid(ii, jj, nx)] == 1.0 || f_ice[cid(ii, jp1, nx)] == 1.0;
}

// The six faces of a cell's 2D quadrature and their weights in the cell value.
// acx: faces (im1 | i) x (jm1 | j | jp1); corner SW takes (im1, jm1) and (im1, j),
// SE (i, jm1) and (i, j), NE (i, j) and (i, jp1), NW (im1, j) and (im1, jp1), each
// the mean of its active faces; the cell value is the mean of the four corners.
struct Quad6 {
    int f[6];
    double w[6];
    YG_DEV double at(const double* v) const {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 6; q++)
            if (w[q] != 0.0) s = fma(w[q], v[f[q]], s);
        return s;
    }
};

// corners given as pairs of entries of the face list
YG_DEV void quad6_weights(Quad6& Q, const bool a[6], const int pairs[4][2]) {
#pragma unroll
    for (int q = 0; q < 6; q++) Q.w[q] = 0.0;
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const int p0 = pairs[c][0], p1 = pairs[c][1];
        const int n = (int)a[p0] + (int)a[p1];
        if (n == 0) continue;
        const double w = 0.25 / (double)n;
        if (a[p0]) Q.w[p0] += w;
        if (a[p1]) Q.w[p1] += w;
    }
}

// acx quadrature of cell (i, j): faces 0..2 = (im1, jm1 | j | jp1), 3..5 = (i, ...)
YG_DEV Quad6 quad_acx(const double* f_ice, int i, int j, int im1, int jm1, int jp1, int nx, int ny, int bc) {
    Quad6 Q;
    const int js[3] = {jm1, j, jp1};
    bool a[6];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        Q.f[r] = cid(im1, js[r], nx);
        Q.f[3 + r] = cid(i, js[r], nx);
        a[r] = act_x(f_ice, im1, js[r], nx, ny, bc);
        a[3 + r] = act_x(f_ice, i, js[r], nx, ny, bc);
    }
    const int pairs[4][2] = {{0, 1}, {3, 4}, {4, 5}, {1, 2}};   // SW, SE, NE, NW
    quad6_weights(Q, a, pairs);
    return Q;
}

// acy quadrature of cell (i, j): faces 0..2 = (im1 | i | ip1, jm1), 3..5 = (..., j);
// corner SW takes (im1, jm1) and (i, jm1), SE (i, jm1) and (ip1, jm1), NE (i, j)
// and (ip1, j), NW (im1, j) and (i, j)
YG_DEV Quad6 quad_acy(const double* f_ice, int i, int j, int im1, int ip1, int jm1, int nx, int ny, int bc) {
    Quad6 Q;
    const int is[3] = {im1, i, ip1};
    bool a[6];
#pragma unroll
    for (int r = 0; r < 3; r++) {
        Q.f[r] = cid(is[r], jm1, nx);
        Q.f[3 + r] = cid(is[r], j, nx);
        a[r] = act_y(f_ice, is[r], jm1, nx, ny, bc);
        a[3 + r] = act_y(f_ice, is[r], j, nx, ny, bc);
    }
    const int pairs[4][2] = {{0, 1}, {1, 2}, {4, 5}, {3, 4}};
    quad6_weights(Q, a, pairs);
    return Q;
}

// 2D quadrature of a field on the cell centres: each corner the mean of its four
// cells, the cell value the mean of the corners (weights over the 3 x 3 block)
struct Quad9 {
    int f[9];
    double w[9];
    YG_DEV double at(const double* v) const {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < 9; q++) s = fma(w[q], v[f[q]], s);
        return s;
    }
};
YG_DEV Quad9 quad_aa(int i, int j, int im1, int ip1, int jm1, int jp1, int nx) {
    Quad9 Q;
    const int is[3] = {im1, i, ip1}, js[3] = {jm1, j, jp1};
    const double wt[3] = {0.25, 0.5, 0.25};
#pragma unroll
    for (int b = 0; b < 3; b++)
#pragma unroll
        for (int a = 0; a < 3; a++) {
            Q.f[a + 3 * b] = cid(is[a], js[b], nx);
            Q.w[a + 3 * b] = wt[a] * wt[b];
        }
    return Q;
}

// dudx and dvdy of calc_strain_rate_horizontal_2D (deformation.f90:1393-1507) at
// face (ii, jj) of one layer: centred, one-sided second order at ice margins, first
// order where the second neighbour is the clamped edge
YG_DEV double dudx_face(const double* ux, const double* f_ice, int ii, int jj, int nx, int ny, int bc, double dx) {
    int im1, ip1, jm1, jp1;
    nbr_bc(ii, jj, nx, ny, bc, im1, ip1, jm1, jp1);
    const int c = cid(ii, jj, nx), cm = cid(im1, jj, nx), cp = cid(ip1, jj, nx);
    const double f0 = f_ice[c], fp = f_ice[cp];
    if (f0 == 1.0 && fp < 1.0) {
        int im2, t1, t2, t3;
        nbr_bc(im1, jj, nx, ny, bc, im2, t1, t2, t3);
        if (f_ice[cm] == 1.0 && im2 != im1)
            return (ux[cid(im2, jj, nx)] - 4.0 * ux[cm] + 3.0 * ux[c]) / (2.0 * dx);
        return (ux[c] - ux[cm]) / dx;
    }
    if (f0 < 1.0 && fp == 1.0) {
        int t0, ip2, t2, t3;
        nbr_bc(ip1, jj, nx, ny, bc, t0, ip2, t2, t3);
        if (ip2 != ip1 && f_ice[cid(ip2, jj, nx)] == 1.0)
            return -(ux[cid(ip2, jj, nx)] - 4.0 * ux[cp] + 3.0 * ux[c]) / (2.0 * dx);
        return (ux[cp] - ux[c]) / dx;
    }
    return (ux[cp] - ux[cm]) / (2.0 * dx);
}
YG_DEV double dvdy_face(const double* uy, const double* f_ice, int ii, int jj, int nx, int ny, int bc, double dy) {
    int im1, ip1, jm1, jp1;
    nbr_bc(ii, jj, nx, ny, bc, im1, ip1, jm1, jp1);
    const int c = cid(ii, jj, nx), cm = cid(ii, jm1, nx), cp = cid(ii, jp1, nx);
    const double f0 = f_ice[c], fp = f_ice[cp];
    if (f0 == 1.0 && fp < 1.0) {
        int t0, t1, jm2, t3;
        nbr_bc(ii, jm1, nx, ny, bc, t0, t1, jm2, t3);
        if (f_ice[cm] == 1.0 && jm2 != jm1)
            return (uy[cid(ii, jm2, nx)] - 4.0 * uy[cm] + 3.0 * uy[c]) / (2.0 * dy);
        return (uy[c] - uy[cm]) / dy;
    }
    if (f0 < 1.0 && fp == 1.0) {
        int t0, t1, t2, jp2;
        nbr_bc(ii, jp1, nx, ny, bc, t0, t1, t2, jp2);
        if (jp2 != jp1 && f_ice[cid(ii, jp2, nx)] == 1.0)
            return -(uy[cid(ii, jp2, nx)] - 4.0 * uy[cp] + 3.0 * uy[c]) / (2.0 * dy);
        return (uy[cp] - uy[c]) / dy;
    }
    return (uy[cp] - uy[cm]) / (2.0 * dy);
}

// the quadrature of the per-layer strain rate: the strain rate is evaluated at the
// faces with a non-zero weight only
YG_DEV double quad_dudx(const Quad6& Q, const double* ux, const double* f_ice, int nx, int ny, int bc, double dx) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 6; q++)
        if (Q.w[q] != 0.0) {
            const int ii = Q.f[q] % nx, jj = Q.f[q] / nx;
            s = fma(Q.w[q], dudx_face(ux, f_ice, ii, jj, nx, ny, bc, dx), s);
        }
    return s;
}
YG_DEV double quad_dvdy(const Quad6& Q, const double* uy, const double* f_ice, int nx, int ny, int bc, double dy) {
    double s = 0.0;
#pragma unroll
    for (int q = 0; q < 6; q++)
        if (Q.w[q] != 0.0) {
            const int ii = Q.f[q] % nx, jj = Q.f[q] / nx;
            s = fma(Q.w[q], dvdy_face(uy, f_ice, ii, jj, nx, ny, bc, dy), s);
        }
    return s;
}

}  // namespace

// uz_method 2 (jac = false) and 3 (jac = true), 0-based: ac level kc, aa layer ka
__global__ void __launch_bounds__(256) k_uz3d_quad(ygpu_uz3d U, int bc, bool jac) {
    const int nx = U.nx, ny = U.ny, nza = U.nz_aa, nzc = U.nz_ac;
    const size_t n2 = (size_t)nx * ny;
    const double f_bmb = U.use_bmb ? 1.0 : 0.0;
    const double* za = U.zeta_aa;
    const double* zc = U.zeta_ac;
    for (int cc = blockIdx.x * blockDim.x + threadIdx.x; cc < nx * ny; cc += gridDim.x * blockDim.x) {
        const int i = cc % nx, j = cc / nx;
        const size_t c = cc;
        const double dzbdt = U.dzbdt[c], dzsdt = U.dzsdt[c];
        if (!(U.f_ice[c] == 1.0)) {
            const double u = flush15(dzbdt - fmax(U.smb[c], 0.0));
            for (int kc = 0; kc < nzc; kc++) {
                U.uz[(size_t)kc * n2 + c] = u;
                U.uz_star[(size_t)kc * n2 + c] = u;
            }
            if (U.uz_srf_err) U.uz_srf_err[c] = 0.0;
            continue;
        }
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        const Quad6 QX = quad_acx(U.f_ice, i, j, im1, jm1, jp1, nx, ny, bc);
        const Quad6 QY = quad_acy(U.f_ice, i, j, im1, ip1, jm1, nx, ny, bc);
        const double H = U.H_ice[c], H_inv = 1.0 / H;
        const double bx = QX.at(U.dzbdx), by = QY.at(U.dzbdy), sx = QX.at(U.dzsdx), sy = QY.at(U.dzsdy);
        auto MX = [&](int k) { return QX.at(U.ux + (size_t)k * n2); };
        auto MY = [&](int k) { return QY.at(U.uy + (size_t)k * n2); };
        // basal value, Greve and Blatter (2009) Eq. 5.31
        double uz = flush15(dzbdt + 0.0 + f_bmb * U.bmb[c] + MX(0) * bx + MY(0) * by);
        U.uz[c] = uz;
        // 2D values of the layers below, at and above the current one (method 3:
        // jac_dxx, jac_dyy; the 1-2-1 mean is the 3D value)
        double wx_m = 0.0, wx_0 = 0.0, wx_p = 0.0, wy_m = 0.0, wy_0 = 0.0, wy_p = 0.0;
        if (jac) {
            wx_0 = QX.at(U.jac_dxx);
            wy_0 = QY.at(U.jac_dyy);
            wx_m = wx_0;
            wy_m = wy_0;
            wx_p = nza > 1 ? QX.at(U.jac_dxx + n2) : wx_0;
            wy_p = nza > 1 ? QY.at(U.jac_dyy + n2) : wy_0;
        }
        for (int kc = 1; kc < nzc; kc++) {
            double div;
            if (jac) {
                // layer kmid = kc - 1 (:218-233): window (kmid-1, kmid, kmid+1), clamped
                div = 0.25 * (wx_m + 2.0 * wx_0 + wx_p) + 0.25 * (wy_m + 2.0 * wy_0 + wy_p);
                const int knext = kc + 1 < nza ? kc + 1 : nza - 1;   // layer above the next kmid
                wx_m = wx_0; wy_m = wy_0;
                wx_0 = wx_p; wy_0 = wy_p;
                if (kc < nzc - 1) {
                    wx_p = QX.at(U.jac_dxx + (size_t)knext * n2);
                    wy_p = QY.at(U.jac_dyy + (size_t)knext * n2);
                }
            } else {
                // :535-579: the sigma-corrected layer divergence
                const double z = za[kc - 1];
                const double c_x = -H_inv * ((1.0 - z) * bx + z * sx);
                const double c_y = -H_inv * ((1.0 - z) * by + z * sy);
                int kup, kdn;
                if (kc == 1) { kup = 1; kdn = 0; }
                else if (kc == nzc - 1) { kup = kc - 1; kdn = kc - 2; }
                else { kup = kc; kdn = kc - 2; }
                const double rdz = 1.0 / (za[kup] - za[kdn]);
                const double dudz = (MX(kup) - MX(kdn)) * rdz, dvdz = (MY(kup) - MY(kdn)) * rdz;
                const size_t o = (size_t)(kc - 1) * n2;
                div = fma(c_x, dudz, quad_dudx(QX, U.ux + o, U.f_ice, nx, ny, bc, U.dx)) +
                      fma(c_y, dvdz, quad_dvdy(QY, U.uy + o, U.f_ice, nx, ny, bc, U.dy));
            }
            // Greve and Blatter (2009) Eq. 5.95
            uz = flush15(uz - H * (zc[kc] - zc[kc - 1]) * div);
            U.uz[(size_t)kc * n2 + c] = uz;
        }
        // uz_star, Greve and Blatter (2009) Eq. 5.148 (no 1/H)
        double top = 0.0;
        double mx_lo = MX(0), my_lo = MY(0);
        for (int kc = 0; kc < nzc; kc++) {
            double ux_aa, uy_aa;
            if (kc == 0) { ux_aa = mx_lo; uy_aa = my_lo; }
            else if (kc == nzc - 1) { ux_aa = mx_lo; uy_aa = my_lo; }
            else {
                const double mx_hi = MX(kc), my_hi = MY(kc);
                ux_aa = 0.5 * (mx_hi + mx_lo);
                uy_aa = 0.5 * (my_hi + my_lo);
                mx_lo = mx_hi;
                my_lo = my_hi;
            }
            const double z = zc[kc];
            const double c_x = -((1.0 - z) * bx + z * sx);
            const double c_y = -((1.0 - z) * by + z * sy);
            const double c_t = -((1.0 - z) * dzbdt + z * dzsdt);
            const size_t o = (size_t)kc * n2 + c;
            const double us = flush15(U.uz[o] + ux_aa * c_x + uy_aa * c_y + c_t);
            U.uz_star[o] = us;
            top = us;
        }
        if (U.uz_srf_err) U.uz_srf_err[c] = top + U.smb[c];
    }
}

// calc_strain_rate_tensor_jac_quad3D (deformation.f90:963-1183), 0-based layer k
__global__ void __launch_bounds__(256) k_strain3d(ygpu_strain3d S, int bc) {
    const int nx = S.nx, ny = S.ny, nza = S.nz_aa;
    const size_t n2 = (size_t)nx * ny;
    const double* za = S.zeta_aa;
    for (int cc = blockIdx.x * blockDim.x + threadIdx.x; cc < nx * ny; cc += gridDim.x * blockDim.x) {
        const int i = cc % nx, j = cc / nx;
        const size_t c = cc;
        double* o3[8] = {S.s_dxx, S.s_dyy, S.s_dxy, S.s_dxz, S.s_dyz, S.s_de, S.s_div, S.s_f_shear};
        double* o2[8] = {S.a_dxx, S.a_dyy, S.a_dxy, S.a_dxz, S.a_dyz, S.a_de, S.a_div, S.a_f_shear};
        if (!(S.f_ice[c] == 1.0)) {
            for (int k = 0; k < nza; k++)
#pragma unroll
                for (int q = 0; q < 8; q++) o3[q][(size_t)k * n2 + c] = 0.0;
#pragma unroll
            for (int q = 0; q < 8; q++)
                if (o2[q]) o2[q][c] = 0.0;
            if (S.eps_eig_1) S.eps_eig_1[c] = 0.0;
            if (S.eps_eig_2) S.eps_eig_2[c] = 0.0;
            continue;
        }
        int im1, ip1, jm1, jp1;
        nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
        const Quad6 QX = quad_acx(S.f_ice, i, j, im1, jm1, jp1, nx, ny, bc);
        const Quad6 QY = quad_acy(S.f_ice, i, j, im1, ip1, jm1, nx, ny, bc);
        const Quad9 QA = quad_aa(i, j, im1, ip1, jm1, jp1, nx);
        const bool floating = (S.f_grnd[c] == 0.0);
        // 2D values of the acx / acy fields on layers k-1, k, k+1 (clamped):
        // 0 dxx, 1 dxy, 2 dxz (acx); 3 dyx, 4 dyz, 5 dyy (acy)
        const double* src[6] = {S.dxx, S.dxy, S.dxz, S.dyx, S.dyz, S.dyy};
        double wm[6], w0[6], wp[6];
#pragma unroll
        for (int f = 0; f < 6; f++) {
            const Quad6& Q = (f < 3) ? QX : QY;
            w0[f] = Q.at(src[f]);
            wm[f] = w0[f];
            wp[f] = nza > 1 ? Q.at(src[f] + n2) : w0[f];
        }
        // the cell-centre values of dzx, dzy on the ac level below layer k
        double zx_lo = QA.at(S.dzx), zy_lo = QA.at(S.dzy);
        double prev[8], sum[8];
#pragma unroll
        for (int q = 0; q < 8; q++) { prev[q] = 0.0; sum[q] = 0.0; }
        for (int k = 0; k < nza; k++) {
            double v[6];
#pragma unroll
            for (int f = 0; f < 6; f++) v[f] = 0.25 * (wm[f] + 2.0 * w0[f] + wp[f]);
            const double zx_hi = QA.at(S.dzx + (size_t)(k + 1) * n2), zy_hi = QA.at(S.dzy + (size_t)(k + 1) * n2);
            const double dxx = v[0], dyy = v[5];
            const double dxy = 0.5 * (v[1] + v[3]);
            const double dxz = 0.5 * (v[2] + 0.5 * (zx_lo + zx_hi));
            const double dyz = 0.5 * (v[4] + 0.5 * (zy_lo + zy_hi));
            zx_lo = zx_hi;
            zy_lo = zy_hi;
            double de = sqrt(dxx * dxx + dyy * dyy + dxx * dyy + dxy * dxy + dxz * dxz + dyz * dyz);
            if (de > S.de_max) de = S.de_max;
            double fs = (de > 0.0) ? sqrt(dxz * dxz + dyz * dyz) / de : 1.0;
            if (floating) fs = 0.0;
            fs = fmin(fmax(fs, 0.0), 1.0);
            const double val[8] = {dxx, dyy, dxy, dxz, dyz, de, dxx + dyy, fs};
            const size_t o = (size_t)k * n2 + c;
#pragma unroll
            for (int q = 0; q < 8; q++) {
                o3[q][o] = val[q];
                // trapezoid integral over zeta_aa (integrate_trapezoid1D_pt)
                if (k > 0) sum[q] = fma(0.5 * (val[q] + prev[q]), za[k] - za[k - 1], sum[q]);
                prev[q] = val[q];
            }
            // slide the layer window
            if (k + 1 < nza) {
                const int kn = (k + 2 < nza) ? k + 2 : nza - 1;
#pragma unroll
                for (int f = 0; f < 6; f++) {
                    wm[f] = w0[f];
                    w0[f] = wp[f];
                    const Quad6& Q = (f < 3) ? QX : QY;
                    wp[f] = Q.at(src[f] + (size_t)kn * n2);
                }
            }
        }
#pragma unroll
        for (int q = 0; q < 8; q++)
            if (o2[q]) o2[q][c] = sum[q];
        if (S.eps_eig_1 && S.eps_eig_2) {
            // calc_2D_eigen_values (deformation.f90:1542-1595) of the averaged tensor
            const double txx = sum[0], tyy = sum[1], txy = sum[2];
            const double b = -(txx + tyy), cq = txx * tyy - txy * txy;
            double e1 = 0.0, e2 = 0.0;
            if (b * b - 4.0 * cq > 0.0) {
                const double root = sqrt(b * b - 4.0 * cq);
                const double l1 = (-b + root) * 0.5, l2 = (-b - root) * 0.5;
                e1 = l1 > l2 ? l1 : l2;
                e2 = l1 > l2 ? l2 : l1;
            }
            S.eps_eig_1[c] = e1;
            S.eps_eig_2[c] = e2;
        }
    }
}

static int post_grid(int n) {
    int g = (n + 255) / 256;
    return g < 1 ? 1 : (g > 65535 ? 65535 : g);
}

int ygpu_uz3d_quad_device(cudaStream_t s, const ygpu_uz3d& U, int bc, int method) {
    k_uz3d_quad<<<post_grid(U.nx * U.ny), 256, 0, s>>>(U, bc, method == YGPU_UZ_JAC);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("vertical velocity (quadrature) kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

int ygpu_strain3d_device(cudaStream_t s, const ygpu_strain3d& S, int bc) {
    k_strain3d<<<post_grid(S.nx * S.ny), 256, 0, s>>>(S, bc);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ygpu_set_error("strain-rate tensor kernel: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}
