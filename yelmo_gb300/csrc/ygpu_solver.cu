// ygpu_solver.cu -- the persistent SSA/DIVA Picard solver for sm_103a.
//
// One cooperative launch solves a batch of instances. The launch is split
// into teams of CTAs; a team takes an instance from a device work queue and
// runs its whole Picard loop (calc_velocity_ssa, velocity_ssa.f90:60-357, and
// calc_velocity_diva, velocity_diva.f90:59-429) without returning to the
// host, then takes the next instance. Phases inside a team are separated by
// team barriers (bounded spin waits); dot products and norms are deterministic
// team all-reduces. A single large instance is one team spanning the grid.
//
// Phases of one Picard iteration:
//   strain      horizontal strain rates on the faces (calc_strain_rate_horizontal_2D)
//   column      3D viscosity (nodes/aa), log relaxation, depth integrals visc_eff_int
//               and F2, basal friction beta on aa-nodes, all in one pass over each column
//   faces       staggered F2 and beta, beta_eff, beta_min, speed-limit drag, N_ab,
//               operator drag coefficients
//   system      right-hand side, start vector and Jacobi diagonal of the
//               matrix-free residual or energy operator
//   krylov      CG / BiCGSTAB, FP64, or FP32 inside FP64 defect correction
//   epilogue    velocity extraction, clip, relaxation, L2 convergence norm,
//               error matrix, basal stress and basal velocity
#include <cuda_runtime.h>
#include <stdlib.h>
#include <string.h>
#include <vector>
#include <mutex>
#include <atomic>

#include <math.h>
#include <stdio.h>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

// 2x2 Gauss-Legendre weights of the bilinear corner interpolation, node q
// (SW, SE, NE, NW) from corner c (same order); set by the host.
__constant__ double c_gqw[4][4];
__constant__ float c_gqwf[4][4];   // the same weights rounded to FP32

static const double TOL_UNDERFLOW = 1e-15;
#define VISC_MIN 1e5

// ---------------------------------------------------------------------------
// Per-solve constants derived once from the instance and the parameters
// ---------------------------------------------------------------------------
struct Geo {
    int nx, ny, nz, n2, nu, bc;
    unsigned bb;                   // border_bits
    bool per_x, per_y;             // energy assembler periodicity (both sides)
    double dx, dy, dxdy, dyodx, dxody;
};

YG_DEV Geo make_geo(const Inst& I, const ygpu_dyn_par& P) {
    Geo G;
    G.nx = I.nx; G.ny = I.ny; G.nz = I.nz; G.n2 = I.n2; G.nu = I.nu; G.bc = P.boundaries;
    G.bb = border_bits(P.boundaries);
    G.per_x = bper(G.bb, 0) && bper(G.bb, 2);
    G.per_y = bper(G.bb, 1) && bper(G.bb, 3);
    G.dx = I.dx; G.dy = I.dy; G.dxdy = I.dx * I.dy; G.dyodx = I.dy / I.dx; G.dxody = I.dx / I.dy;
    return G;
}

// Grid constants of the operators in the arithmetic T, converted once per
// solve instead of once per row (a double -> float conversion runs on the FP64
// pipe).
template <typename T>
struct OpK {
    T dyodx, dxody, inv_dx, inv_dy, inv_dxdx, inv_dydy, inv_dxdy;
};
template <typename T>
YG_DEV OpK<T> make_opk(const Geo& G) {
    OpK<T> K;
    K.dyodx = (T)G.dyodx;
    K.dxody = (T)G.dxody;
    K.inv_dx = T(1.0 / G.dx);
    K.inv_dy = T(1.0 / G.dy);
    K.inv_dxdx = T(1.0 / (G.dx * G.dx));
    K.inv_dydy = T(1.0 / (G.dy * G.dy));
    K.inv_dxdy = T(1.0 / (G.dx * G.dy));
    return K;
}

// ---------------------------------------------------------------------------
// Quadrature helpers (restated gq2D_to_nodes_*, see the oracle for the rule)
// ---------------------------------------------------------------------------
template <typename V>
YG_DEV V gq_weight(int q, int c);
template <>
YG_DEV double gq_weight<double>(int q, int c) { return c_gqw[q][c]; }
template <>
YG_DEV float gq_weight<float>(int q, int c) { return c_gqwf[q][c]; }

template <typename V>
YG_DEV void gq_nodes(const V c[4], V v[4]) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
        V s = gq_weight<V>(q, 0) * c[0];
        s = s + gq_weight<V>(q, 1) * c[1];
        s = s + gq_weight<V>(q, 2) * c[2];
        s = s + gq_weight<V>(q, 3) * c[3];
        v[q] = s;
    }
}
YG_DEV double gq_mean(const double v[4]) { return (((v[0] + v[1]) + v[2]) + v[3]) / 4.0; }

// Means over the active values. Division by the count 1, 2 or 4 is written as
// an exact scaling (same result, no division); only a count of 3 divides.
template <typename V>
YG_DEV V mean2_act(V a, V b, bool aa, bool ab) {
    const V s = (aa ? a : V(0)) + (ab ? b : V(0));
    return (aa && ab) ? s * V(0.5) : s;
}
template <typename V>
YG_DEV V mean4_act(V a, V b, V c, V d, bool aa, bool ab, bool ac, bool ad) {
    int n = (int)aa + (int)ab + (int)ac + (int)ad;
    if (n == 0) return V(0);
    V s = (aa ? a : V(0)) + (ab ? b : V(0));
    s = s + (ac ? c : V(0));
    s = s + (ad ? d : V(0));
    if (n == 4) return s * V(0.25);
    if (n == 2) return s * V(0.5);
    if (n == 1) return s;
    return s / V(3);
}

// neighbourhood of a cell: index of (im1|i|ip1, jm1|j|jp1)
struct Nb {
    int i, j, im1, ip1, jm1, jp1;
};
YG_DEV Nb make_nb(const Geo& G, int c) {
    Nb n;
    n.i = c % G.nx;
    n.j = c / G.nx;
    nbr_bc(n.i, n.j, G.nx, G.ny, G.bc, n.im1, n.ip1, n.jm1, n.jp1);
    return n;
}
#define CI(ii, jj) ((ii) + G.nx * (jj))

// active faces (calc_active_faces, deformation.f90:1316-1344)
// Per-cell flags of a solve's fixed inputs (Inst::cflag, set once by the setup
// step): the phases test these bits instead of comparing FP64 fields, whose
// compares run on the slow FP64 pipe of this part.
#define CF_ICE 1u      // f_ice == 1
#define CF_ACTX 2u     // x face active: f_ice == 1 on either side (acx ice mask)
#define CF_ACTY 4u     // y face active
#define CF_OCN 8u      // ice-free and z_bed < z_sl
#define CF_PART 16u    // f_ice < 1
#define CF_G0 32u      // f_grnd == 0
#define CF_GPOS 64u    // f_grnd > 0
YG_DEV unsigned char cell_flags(const Geo& G, const Inst& I, int c) {
    const Nb n = make_nb(G, c);
    const bool ice = (I.f_ice[c] == 1.0);
    unsigned fl = ice ? CF_ICE : 0u;
    if (ice || I.f_ice[CI(n.ip1, n.j)] == 1.0) fl |= CF_ACTX;
    if (ice || I.f_ice[CI(n.i, n.jp1)] == 1.0) fl |= CF_ACTY;
    if (!ice && I.z_bed[c] < I.z_sl[c]) fl |= CF_OCN;
    if (I.f_ice[c] < 1.0) fl |= CF_PART;
    if (I.f_grnd[c] == 0.0) fl |= CF_G0;
    if (I.f_grnd[c] > 0.0) fl |= CF_GPOS;
    return (unsigned char)fl;
}
// calc_staggered_margin (velocity_diva.f90:1052-1082) with the f_ice tests read
// from the cell flags of the two cells (the same compares, made by the setup step)
template <typename T>
YG_DEV T stag_margin_fl(T v0, T v1, unsigned f0, unsigned f1) {
    if ((f0 & CF_ICE) && (f1 & CF_PART)) return v0;
    if ((f0 & CF_PART) && (f1 & CF_ICE)) return v1;
    return T(0.5) * (v0 + v1);
}
YG_DEV bool act_x(const Geo& G, const unsigned char* fl, int i, int j) { return (fl[CI(i, j)] & CF_ACTX) != 0; }
YG_DEV bool act_y(const Geo& G, const unsigned char* fl, int i, int j) { return (fl[CI(i, j)] & CF_ACTY) != 0; }

// acx-field to quadrature nodes of cell nb (corner = mean of the acx faces above/below)
template <typename F, typename V>
YG_DEV void nodes_acx(const Geo& G, const Nb& n, F val, const bool* ax, V v[4]) {
    // ax: active flags of faces [im1,jm1],[im1,j],[im1,jp1],[i,jm1],[i,j],[i,jp1]
    V c[4];
    V a_im1_jm1 = (V)val(n.im1, n.jm1), a_im1_j = (V)val(n.im1, n.j), a_im1_jp1 = (V)val(n.im1, n.jp1);
    V a_i_jm1 = (V)val(n.i, n.jm1), a_i_j = (V)val(n.i, n.j), a_i_jp1 = (V)val(n.i, n.jp1);
    if (ax) {
        c[0] = mean2_act(a_im1_jm1, a_im1_j, ax[0], ax[1]);
        c[1] = mean2_act(a_i_jm1, a_i_j, ax[3], ax[4]);
        c[2] = mean2_act(a_i_j, a_i_jp1, ax[4], ax[5]);
        c[3] = mean2_act(a_im1_j, a_im1_jp1, ax[1], ax[2]);
    } else {
        c[0] = V(0.5) * (a_im1_jm1 + a_im1_j);
        c[1] = V(0.5) * (a_i_jm1 + a_i_j);
        c[2] = V(0.5) * (a_i_j + a_i_jp1);
        c[3] = V(0.5) * (a_im1_j + a_im1_jp1);
    }
    gq_nodes(c, v);
}
// acy-field to nodes (corner = mean of the acy faces left/right)
template <typename F, typename V>
YG_DEV void nodes_acy(const Geo& G, const Nb& n, F val, const bool* ay, V v[4]) {
    // ay: active flags of faces [im1,jm1],[i,jm1],[ip1,jm1],[im1,j],[i,j],[ip1,j]
    V c[4];
    V a_im1_jm1 = (V)val(n.im1, n.jm1), a_i_jm1 = (V)val(n.i, n.jm1), a_ip1_jm1 = (V)val(n.ip1, n.jm1);
    V a_im1_j = (V)val(n.im1, n.j), a_i_j = (V)val(n.i, n.j), a_ip1_j = (V)val(n.ip1, n.j);
    if (ay) {
        c[0] = mean2_act(a_im1_jm1, a_i_jm1, ay[0], ay[1]);
        c[1] = mean2_act(a_i_jm1, a_ip1_jm1, ay[1], ay[2]);
        c[2] = mean2_act(a_i_j, a_ip1_j, ay[4], ay[5]);
        c[3] = mean2_act(a_im1_j, a_i_j, ay[3], ay[4]);
    } else {
        c[0] = V(0.5) * (a_im1_jm1 + a_i_jm1);
        c[1] = V(0.5) * (a_i_jm1 + a_ip1_jm1);
        c[2] = V(0.5) * (a_i_j + a_ip1_j);
        c[3] = V(0.5) * (a_im1_j + a_i_j);
    }
    gq_nodes(c, v);
}
// aa-field to nodes (corner = mean of the 4 cells around it; act: active cells only)
template <typename F, typename A>
YG_DEV void nodes_aa(const Geo& G, const Nb& n, F val, A act, bool use_act, double v[4]) {
    const int ii[4][4] = {{n.im1, n.i, n.im1, n.i}, {n.i, n.ip1, n.i, n.ip1}, {n.i, n.ip1, n.i, n.ip1}, {n.im1, n.i, n.im1, n.i}};
    const int jj[4][4] = {{n.jm1, n.jm1, n.j, n.j}, {n.jm1, n.jm1, n.j, n.j}, {n.j, n.j, n.jp1, n.jp1}, {n.j, n.j, n.jp1, n.jp1}};
    double c[4];
#pragma unroll
    for (int q = 0; q < 4; q++) {
        double a0 = val(ii[q][0], jj[q][0]), a1 = val(ii[q][1], jj[q][1]);
        double a2 = val(ii[q][2], jj[q][2]), a3 = val(ii[q][3], jj[q][3]);
        if (use_act) {
            c[q] = mean4_act(a0, a1, a2, a3, act(ii[q][0], jj[q][0]), act(ii[q][1], jj[q][1]),
                             act(ii[q][2], jj[q][2]), act(ii[q][3], jj[q][3]));
        } else {
            double s = a0 + a1;
            s = s + a2;
            s = s + a3;
            c[q] = 0.25 * s;
        }
    }
    gq_nodes(c, v);
}

// e^(-1/3) for e > 0, the Glen n = 3 viscosity factor. FP32: the library's
// rcbrtf. FP64: an FP32 seed refined by two Newton steps for y^-3 = e,
// y <- y (4 - e y^3) / 3, which square the seed's relative error (about 1e-7)
// each time, down to FP64 rounding, with a dozen FP64 operations on this part's
// slow FP64 pipe.
template <typename R>
YG_DEV R rcbrt_visc(R e);
template <>
YG_DEV float rcbrt_visc<float>(float e) { return rcbrtf(e); }
template <>
YG_DEV double rcbrt_visc<double>(double e) {
    double y = (double)rcbrtf((float)e);
    const double third = 1.0 / 3.0;
    y = y * (4.0 - e * (y * y * y)) * third;
    y = y * (4.0 - e * (y * y * y)) * third;
    return y;
}
// a^(-1/3) for any a: the seeded Newton form where a is a normal FP32 number
// (where the seed is), the library's FP64 rcbrt elsewhere (0, inf, NaN, tiny)
YG_DEV double rcbrt_any(double a) {
    const float af = (float)a;
    if (af >= 1.17549435e-38f && af <= 3.4e38f) return rcbrt_visc<double>(a);
    return rcbrt(a);
}

// ---------------------------------------------------------------------------
// Phase: horizontal strain rates at the faces of every cell
// (calc_strain_rate_horizontal_2D, deformation.f90:1393-1507)
// ---------------------------------------------------------------------------
// Quotient of an FP64 difference by a grid step: FP64 results divide as the
// reference does; FP32 results (the mixed mode) scale the FP64 difference by
// the FP32 reciprocal, with no FP64 division (a long chain on this part's FP64
// pipe, which runs at about 1/64 of the FP32 rate)
template <typename SD>
YG_DEV SD quot_h(double num, double h, float inv_h) {
    if constexpr (sizeof(SD) == sizeof(float)) return (float)num * inv_h;
    else return num / h;
}
template <typename SD>
YG_DEV SD deriv_active(double vm, double v0, double vp, bool am, bool ap, double h, float inv_h, float inv_2h) {
    if (am && ap) return quot_h<SD>(vp - vm, 2.0 * h, inv_2h);
    if (ap) return quot_h<SD>(vp - v0, h, inv_h);
    if (am) return quot_h<SD>(v0 - vm, h, inv_h);
    return SD(0);
}

template <typename SD>
__device__ __noinline__ void phase_strain(const Inst& I, const Geo& Gr, Team& T, const double* ux, const double* uy, SD* sdudx,
                                          SD* sdudy, SD* sdvdx, SD* sdvdy) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const Geo G = Gr;
    const int tid = t_tid, nthr = t_nthr;
    const unsigned char* fl = I.cflag;
    const double dx = G.dx, dy = G.dy;
    const float ix = (float)(1.0 / dx), iy = (float)(1.0 / dy), i2x = (float)(1.0 / (2.0 * dx)),
                i2y = (float)(1.0 / (2.0 * dy));
    for (int c = tid; c < G.n2; c += nthr) {
        Nb n = make_nb(G, c);
        const int i = n.i, j = n.j;
        SD dudx = quot_h<SD>(ux[CI(n.ip1, j)] - ux[CI(n.im1, j)], 2.0 * dx, i2x);
        SD dudy = deriv_active<SD>(ux[CI(i, n.jm1)], ux[c], ux[CI(i, n.jp1)], act_x(G, fl, i, n.jm1), act_x(G, fl, i, n.jp1),
                                   dy, iy, i2y);
        SD dvdx = deriv_active<SD>(uy[CI(n.im1, j)], uy[c], uy[CI(n.ip1, j)], act_y(G, fl, n.im1, j), act_y(G, fl, n.ip1, j),
                                   dx, ix, i2x);
        SD dvdy = quot_h<SD>(uy[CI(i, n.jp1)] - uy[CI(i, n.jm1)], 2.0 * dy, i2y);
        int d1, d2, d3;
        if ((fl[c] & CF_ICE) && !(fl[CI(n.ip1, j)] & CF_ICE)) {
            int im2;
            nbr_bc(n.im1, j, G.nx, G.ny, G.bc, im2, d1, d2, d3);
            if ((fl[CI(n.im1, j)] & CF_ICE) && im2 != n.im1)
                dudx = quot_h<SD>(1.0 * ux[CI(im2, j)] - 4.0 * ux[CI(n.im1, j)] + 3.0 * ux[c], 2.0 * dx, i2x);
            else
                dudx = quot_h<SD>(ux[c] - ux[CI(n.im1, j)], dx, ix);
        } else if (!(fl[c] & CF_ICE) && (fl[CI(n.ip1, j)] & CF_ICE)) {
            int ip2;
            nbr_bc(n.ip1, j, G.nx, G.ny, G.bc, d1, ip2, d2, d3);
            if (ip2 != n.ip1 && (fl[CI(ip2, j)] & CF_ICE))
                dudx = quot_h<SD>(-(1.0 * ux[CI(ip2, j)] - 4.0 * ux[CI(n.ip1, j)] + 3.0 * ux[c]), 2.0 * dx, i2x);
            else
                dudx = quot_h<SD>(ux[CI(n.ip1, j)] - ux[c], dx, ix);
        }
        if ((fl[c] & CF_ICE) && !(fl[CI(i, n.jp1)] & CF_ICE)) {
            int jm2;
            nbr_bc(i, n.jm1, G.nx, G.ny, G.bc, d1, d2, jm2, d3);
            if ((fl[CI(i, n.jm1)] & CF_ICE) && jm2 != n.jm1)
                dvdy = quot_h<SD>(1.0 * uy[CI(i, jm2)] - 4.0 * uy[CI(i, n.jm1)] + 3.0 * uy[c], 2.0 * dy, i2y);
            else
                dvdy = quot_h<SD>(uy[c] - uy[CI(i, n.jm1)], dy, iy);
        } else if (!(fl[c] & CF_ICE) && (fl[CI(i, n.jp1)] & CF_ICE)) {
            int jp2;
            nbr_bc(i, n.jp1, G.nx, G.ny, G.bc, d1, d2, d3, jp2);
            if (jp2 != n.jp1 && (fl[CI(i, jp2)] & CF_ICE))
                dvdy = quot_h<SD>(-(1.0 * uy[CI(i, jp2)] - 4.0 * uy[CI(i, n.jp1)] + 3.0 * uy[c]), 2.0 * dy, i2y);
            else
                dvdy = quot_h<SD>(uy[CI(i, n.jp1)] - uy[c], dy, iy);
        }
        sdudx[c] = dudx;
        sdudy[c] = dudy;
        sdvdx[c] = dvdx;
        sdvdy[c] = dvdy;
    }
}

// ---------------------------------------------------------------------------
// Basal friction on aa-nodes (calc_beta, basal_dragging.f90:384-579)
// ---------------------------------------------------------------------------
YG_DEV double beta_raw(const Inst& I, const ygpu_dyn_par& P, const Geo& G, int i, int j, const double* ux_b,
                       const double* uy_b) {
    const int m = P.beta_method;
    const int c = CI(i, j);
    double beta;
    if (m == 0) {
        beta = P.beta_const;
    } else {
        const double q = (m == 1) ? 1.0 : P.beta_q;
        const double u0 = P.beta_u0;
        const bool coulomb = (m == 3 || m == 5);
        const bool simple = (m == 4 || m == 5);
        const double ub_min = 1e-3, ub_sq_min = ub_min * ub_min;
        if (I.f_ice[c] == 1.0) {
            Nb n = make_nb(G, c);
            double cbn[4], uxn[4], uyn[4], bn[4];
            if (simple) {
                double ucx = 0.5 * (ux_b[c] + ux_b[CI(n.im1, j)]);
                double ucy = 0.5 * (uy_b[c] + uy_b[CI(i, n.jm1)]);
#pragma unroll
                for (int k = 0; k < 4; k++) { cbn[k] = I.c_bed[c]; uxn[k] = ucx; uyn[k] = ucy; }
            } else {
                auto cb = [&](int a, int b) { return I.c_bed[CI(a, b)]; };
                auto aa = [&](int a, int b) { return I.f_ice[CI(a, b)] == 1.0 && I.f_grnd[CI(a, b)] > 0.0; };
                nodes_aa(G, n, cb, aa, true, cbn);
                bool ax[6] = {act_x(G, I.cflag, n.im1, n.jm1), act_x(G, I.cflag, n.im1, n.j), act_x(G, I.cflag, n.im1, n.jp1),
                              act_x(G, I.cflag, n.i, n.jm1), act_x(G, I.cflag, n.i, n.j), act_x(G, I.cflag, n.i, n.jp1)};
                bool ay[6] = {act_y(G, I.cflag, n.im1, n.jm1), act_y(G, I.cflag, n.i, n.jm1), act_y(G, I.cflag, n.ip1, n.jm1),
                              act_y(G, I.cflag, n.im1, n.j), act_y(G, I.cflag, n.i, n.j), act_y(G, I.cflag, n.ip1, n.j)};
                auto vx = [&](int a, int b) { return ux_b[CI(a, b)]; };
                auto vy = [&](int a, int b) { return uy_b[CI(a, b)]; };
                nodes_acx(G, n, vx, ax, uxn);
                nodes_acy(G, n, vy, ay, uyn);
            }
#pragma unroll
            for (int k = 0; k < 4; k++) {
                double s = uxn[k] * uxn[k] + uyn[k] * uyn[k];
                double uxy = sqrt(s + ub_sq_min);
                double fac = coulomb ? pow(uxy / (uxy + u0), q) : pow(uxy / u0, q);
                bn[k] = cbn[k] * fac * (1.0 / uxy);
            }
            beta = gq_mean(bn);
        } else {
            double uxy = ub_min;
            double fac = coulomb ? pow(uxy / (uxy + u0), q) : pow(uxy / u0, q);
            beta = I.c_bed[c] * fac * (1.0 / uxy);
        }
    }
    const double q_frz = (m == 0 || m == 1) ? 1.0 : P.beta_q;
    beta = beta * pow(I.f_slide[c], -q_frz);
    switch (P.beta_gl_scale) {
        case 0: {
            int im1, ip1, jm1, jp1;
            nbr_bc(i, j, G.nx, G.ny, G.bc, im1, ip1, jm1, jp1);
            const double* fg = I.f_grnd;
            if (fg[c] > 0.0 && (fg[CI(im1, j)] == 0.0 || fg[CI(ip1, j)] == 0.0 || fg[CI(i, jm1)] == 0.0 || fg[CI(i, jp1)] == 0.0))
                beta = beta * P.beta_gl_f;
        } break;
        case 1: {
            double hg = I.H_grnd[c] < P.H_grnd_lim ? I.H_grnd[c] : P.H_grnd_lim;
            double f = hg / P.H_grnd_lim;
            if (f < 0.0) f = 0.0;
            beta = beta * f;
        } break;
        case 2: {
            if (I.f_ice[c] > 0.0) {
                double Heff = I.H[c] / I.f_ice[c];
                if (I.f_ice[c] < 1.0) Heff = 0.0;
                double f;
                if (I.z_bed[c] > I.z_sl[c]) f = Heff;
                else {
                    f = Heff - (I.z_sl[c] - I.z_bed[c]) * (P.rho_sw / P.rho_ice);
                    if (f < 0.0) f = 0.0;
                }
                if (Heff > 0.0) f = f / Heff;
                beta = beta * f;
            }
        } break;
        case 3: beta = I.f_grnd[c] * beta; break;
        default: break;
    }
    if (I.f_grnd[c] == 0.0) beta = 0.0;
    return beta;
}

YG_DEV double beta_aa(const Inst& I, const ygpu_dyn_par& P, const Geo& G, int i, int j, const double* ux_b,
                      const double* uy_b) {
    // edge copies of calc_beta (MISMIP3D: left column; infinite/mask: all edges), then beta_min
    int si = i, sj = j;
    if (G.bc == YGPU_BND_MISMIP3D) {
        if (i == 0) si = 1;
    } else if (G.bc == YGPU_BND_INFINITE) {
        if (i == 0) si = 1;
        if (i == G.nx - 1) si = G.nx - 2;
        if (j == 0) sj = 1;
        if (j == G.ny - 1) sj = G.ny - 2;
    }
    double b = beta_raw(I, P, G, si, sj, ux_b, uy_b);
    if (b > 0.0 && b < P.beta_min) b = P.beta_min;
    return b;
}

// ---------------------------------------------------------------------------
// Phase: A^(-1/n) at the quadrature nodes (once per solve; ATT is constant)
// ---------------------------------------------------------------------------
// In the mixed mode the powers are stored as FP32 (attp read as float*); the
// upper half of the array then holds the FP32 shear copies (shear_f32).
__device__ __noinline__ void phase_att_powers(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const int nz = G.nz, n2 = G.n2;
    const double p2 = -1.0 / I.n_glen;
    const bool glen3 = (I.n_glen == 3.0);
    const bool f32 = (P.precision == YGPU_PREC_MIXED);
    float* af = (float*)I.attp;
    for (int c = t_tid; c < n2; c += t_nthr) {
        Nb n = make_nb(G, c);
        for (int k = 0; k < nz; k++) {
            if (P.visc_method == 1) {
                double attn[4];
                auto att = [&](int a, int b) { return I.ATT[(size_t)k * n2 + CI(a, b)]; };
                nodes_aa(G, n, att, [](int, int) { return true; }, false, attn);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const double v = glen3 ? rcbrt_any(attn[q]) : pow(attn[q], p2);
                    const size_t o = ((size_t)q * nz + k) * n2 + c;
                    if (f32) af[o] = (float)v;
                    else I.attp[o] = v;
                }
            } else {
                const double a = I.ATT[(size_t)k * n2 + c];
                const double v = glen3 ? rcbrt_any(a) : pow(a, p2);
                if (f32) af[(size_t)k * n2 + c] = (float)v;
                else I.attp[(size_t)k * n2 + c] = v;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Phase: vertical shear of the iterate on the faces (DIVA), from the basal
// stress and the viscosity at the start of the iteration
// (calc_vertical_shear_3D, velocity_diva.f90:510-571)
// ---------------------------------------------------------------------------
// FP32 copies of the shear (mixed mode): the upper half of the attp array
YG_DEV float* shear_f32(const Inst& I, int axis) {
    const size_t n3 = (size_t)I.nz * I.n2;
    return (float*)I.attp + (4 + axis) * n3;
}

// R = float (mixed mode): FP32 arithmetic into the FP32 copies that the column
// pass reads; the caller's FP64 duxdz / duydz are those floats widened, written
// once by the final passes rather than every iteration
// Per-layer factors of the vertical passes: 1 - zeta(k) and zeta(k) - zeta(k-1).
// FP32 passes read them from a table in shared memory, filled once per call
// (every thread of the CTA constructs it), instead of forming them in FP64 for
// every cell and layer; FP64 passes form them as the reference does.
#define YG_ZTAB 128
template <typename R>
struct ZTab {
    const double* zeta;
    bool tab;
    float* s_o;
    float* s_d;
    YG_DEV ZTab(const double* z, int nz) : zeta(z) {
        __shared__ float so[YG_ZTAB], sd[YG_ZTAB];
        s_o = so;
        s_d = sd;
        tab = (sizeof(R) == sizeof(float)) && nz <= YG_ZTAB;
        if (tab) {
            __syncthreads();       // a previous call's readers are done
            for (int k = threadIdx.x; k < nz; k += blockDim.x) {
                so[k] = (float)(1.0 - z[k]);
                sd[k] = (k > 0) ? (float)(z[k] - z[k - 1]) : 0.0f;
            }
            __syncthreads();
        }
    }
    YG_DEV R omz(int k) const { return tab ? (R)s_o[k] : (R)(1.0 - zeta[k]); }
    YG_DEV R dz(int k) const { return tab ? (R)s_d[k] : (R)(zeta[k] - zeta[k - 1]); }
};

template <typename R, typename VS>
__device__ __noinline__ void phase_shear(const Inst& I, const Geo& Gr, Team& T, const VS* vcur) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const Geo G = Gr;
    const int nz = G.nz, n2 = G.n2;
    float* sx32 = shear_f32(I, 0);
    float* sy32 = shear_f32(I, 1);
    const ZTab<R> zt(I.zeta, nz);
    for (int c = t_tid; c < n2; c += t_nthr) {
        Nb n = make_nb(G, c);
        const int cx = CI(n.ip1, n.j), cy = CI(n.i, n.jp1);
        const R tx = (R)I.taub_x[c], ty = (R)I.taub_y[c];
        const unsigned fc = I.cflag[c], fx = I.cflag[cx], fy = I.cflag[cy];
        for (int k = 0; k < nz; k++) {
            const size_t o = (size_t)k * n2;
            const R omz = zt.omz(k);
            const R vc = (R)vcur[o + c];
            R va = stag_margin_fl<R>(vc, (R)vcur[o + cx], fc, fx);
            const R gx = (va != R(0)) ? (tx / va) * omz : R(0);
            va = stag_margin_fl<R>(vc, (R)vcur[o + cy], fc, fy);
            const R gy = (va != R(0)) ? (ty / va) * omz : R(0);
            if (sizeof(R) == sizeof(float)) {
                sx32[o + c] = (float)gx;
                sy32[o + c] = (float)gy;
            } else {
                I.duxdz[o + c] = (double)gx;
                I.duydz[o + c] = (double)gy;
            }
        }
    }
}

// The layer-independent part of the strain-rate invariant at the four
// quadrature nodes of cell n: the horizontal terms, summed in the reference's
// order (the layer loops add the shear terms and eps_0^2)
template <typename R, typename SR>
YG_DEV void node_strain_invariant(const Geo& G, const Nb& n, const SR* sdudx, const SR* sdudy, const SR* sdvdx,
                                  const SR* sdvdy, const bool* ax, const bool* ay, R eb[4]) {
    R dudxn[4], dudyn[4], dvdxn[4], dvdyn[4];
    nodes_acx(G, n, [&](int a, int b) { return sdudx[CI(a, b)]; }, ax, dudxn);
    nodes_acx(G, n, [&](int a, int b) { return sdudy[CI(a, b)]; }, ax, dudyn);
    nodes_acy(G, n, [&](int a, int b) { return sdvdx[CI(a, b)]; }, ay, dvdxn);
    nodes_acy(G, n, [&](int a, int b) { return sdvdy[CI(a, b)]; }, ay, dvdyn);
#pragma unroll
    for (int q = 0; q < 4; q++) {
        const R sh = dudyn[q] + dvdxn[q];
        R e = dudxn[q] * dudxn[q] + dvdyn[q] * dvdyn[q];
        e = e + dudxn[q] * dvdyn[q];
        eb[q] = e + R(0.25) * (sh * sh);
    }
}

// ---------------------------------------------------------------------------
// Phase: column pass -- viscosity, relaxation, depth integrals, beta (aa)
// R is the arithmetic of the viscosity (double: FP64 solve; float: mixed)
// ---------------------------------------------------------------------------
// VD is the storage of the new viscosity (double, or float for the FP32
// working copy of the mixed mode); log(visc) is kept in R. vcur (the caller's
// FP64 viscosity) is read only when no log is carried yet (first iteration).
template <typename R, typename VD, typename SR = double>
__device__ __noinline__ void phase_column(const Inst& I, const ygpu_dyn_par& P, const Geo& Gr, Team& T,
                                          const double* vcur, VD* vnew, const SR* sdudx,
                                          const SR* sdudy, const SR* sdvdx, const SR* sdvdy, bool relax,
                                          bool diva, bool first_copy, bool have_log, bool visc_only = false) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const Geo G = Gr;
    const int nz = G.nz, n2 = G.n2;
    const R p1 = (R)((1.0 - I.n_glen) / (2.0 * I.n_glen));
    const bool glen3 = (I.n_glen == 3.0);
    const R eps0sq = (R)(P.eps_0 * P.eps_0);
    const R rel = (R)P.ssa_iter_rel;
    const double* zeta = I.zeta;
    const int vm = P.visc_method;
    // A^(-1/n) at the nodes and log(visc): FP32 storage in the mixed mode
    // restrict-qualified: the layer's loads do not wait for the previous layer's stores
    const R* __restrict__ attp_r = (const R*)I.attp;
    R* __restrict__ lv = (R*)I.lvis;
    VD* __restrict__ vn = vnew;
    const R* __restrict__ shx_r = (sizeof(R) == sizeof(float)) ? (const R*)shear_f32(I, 0) : (const R*)I.duxdz;
    const R* __restrict__ shy_r = (sizeof(R) == sizeof(float)) ? (const R*)shear_f32(I, 1) : (const R*)I.duydz;
    const ZTab<R> zt(zeta, nz);
    for (int c = t_tid; c < n2; c += t_nthr) {
        Nb n = make_nb(G, c);
        if (first_copy) {
            I.ux_nm1[c] = I.u_x[c];
            I.uy_nm1[c] = I.u_y[c];
            if (diva) {
                I.tbp_x[c] = I.taub_x[c];
                I.tbp_y[c] = I.taub_y[c];
            }
        }
        const bool ice = (I.cflag[c] & CF_ICE) != 0;
        const double Hc = I.H[c];
        // quadrature nodes: the layer-independent part of the strain-rate invariant
        // (the horizontal terms, summed in the reference's order)
        R eb[4];
        bool ax[6], ay[6];
        R e_aa = R(0);
        if (ice && vm == 1) {
            const unsigned char* fl = I.cflag;
            ax[0] = act_x(G, fl, n.im1, n.jm1); ax[1] = act_x(G, fl, n.im1, n.j); ax[2] = act_x(G, fl, n.im1, n.jp1);
            ax[3] = act_x(G, fl, n.i, n.jm1); ax[4] = act_x(G, fl, n.i, n.j); ax[5] = act_x(G, fl, n.i, n.jp1);
            ay[0] = act_y(G, fl, n.im1, n.jm1); ay[1] = act_y(G, fl, n.i, n.jm1); ay[2] = act_y(G, fl, n.ip1, n.jm1);
            ay[3] = act_y(G, fl, n.im1, n.j); ay[4] = act_y(G, fl, n.i, n.j); ay[5] = act_y(G, fl, n.ip1, n.j);
            node_strain_invariant<R>(G, n, sdudx, sdudy, sdvdx, sdvdy, ax, ay, eb);
        } else if (ice && vm == 2) {
            const double* ux = I.u_x;
            const double* uy = I.u_y;
            const int i = n.i, j = n.j;
            double dudx = (ux[c] - ux[CI(n.im1, j)]) / G.dx;
            double dvdy = (uy[c] - uy[CI(i, n.jm1)]) / G.dy;
            double dudy1 = (ux[CI(i, n.jp1)] - ux[CI(i, n.jm1)]) / (2.0 * G.dy);
            double dudy2 = (ux[CI(n.im1, n.jp1)] - ux[CI(n.im1, n.jm1)]) / (2.0 * G.dy);
            double dudy = 0.5 * (dudy1 + dudy2);
            double dvdx1 = (uy[CI(n.ip1, j)] - uy[CI(n.im1, j)]) / (2.0 * G.dx);
            double dvdx2 = (uy[CI(n.ip1, n.jm1)] - uy[CI(n.im1, n.jm1)]) / (2.0 * G.dx);
            double dvdx = 0.5 * (dvdx1 + dvdx2);
            double sh = dudy + dvdx;
            double e = dudx * dudx + dvdy * dvdy;
            e = e + dudx * dvdy;
            e = e + 0.25 * (sh * sh);
            e_aa = (R)e;
        }
        R vint = R(0), f2 = R(0), vprev = R(0), gprev = R(0);
        const R Hr = (R)Hc;
        for (int k = 0; k < nz; k++) {
            const size_t ck = (size_t)k * n2 + c;
            R v;
            if (vm == 0) {
                v = (R)P.visc_const;
            } else if (!ice) {
                v = (R)VISC_MIN;
            } else if (vm == 1) {
                R dudzn[4], dvdzn[4], vn[4];
                if (diva) {
                    // FP64 mode: the FP64 shear; mixed mode: its FP32 copy
                    const R* __restrict__ dz = shx_r + (size_t)k * n2;
                    const R* __restrict__ dzy = shy_r + (size_t)k * n2;
                    nodes_acx(G, n, [&](int a, int b) { return dz[CI(a, b)]; }, ax, dudzn);
                    nodes_acy(G, n, [&](int a, int b) { return dzy[CI(a, b)]; }, ay, dvdzn);
                }
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    R e = eb[q];
                    if (diva) {
                        e = e + R(0.25) * (dudzn[q] * dudzn[q]);
                        e = e + R(0.25) * (dvdzn[q] * dvdzn[q]);
                    }
                    e = e + eps0sq;
                    R ep = glen3 ? rcbrt_visc<R>(e) : pow(e, p1);
                    vn[q] = R(0.5) * ep * attp_r[((size_t)q * nz + k) * n2 + c];
                }
                v = (((vn[0] + vn[1]) + vn[2]) + vn[3]) / R(4);
            } else {
                R e = e_aa;
                if (diva) {
                    // the FP64 shear, or (mixed) its FP32 copy widened: the same values
                    const size_t o = (size_t)k * n2;
                    const bool f32 = (sizeof(R) == sizeof(float));
                    const float* fx = f32 ? shear_f32(I, 0) + o : nullptr;
                    const float* fy = f32 ? shear_f32(I, 1) + o : nullptr;
                    auto shx = [&](int q) { return f32 ? (double)fx[q] : I.duxdz[o + q]; };
                    auto shy = [&](int q) { return f32 ? (double)fy[q] : I.duydz[o + q]; };
                    R dzx = (R)(0.5 * (shx(c) + shx(CI(n.im1, n.j))));
                    R dzyv = (R)(0.5 * (shy(c) + shy(CI(n.i, n.jm1))));
                    e = e + R(0.25) * (dzx * dzx);
                    e = e + R(0.25) * (dzyv * dzyv);
                }
                e = e + eps0sq;
                R ep = glen3 ? rcbrt_visc<R>(e) : pow(e, p1);
                v = R(0.5) * ep * attp_r[ck];
            }
            R vr;
            if (relax) {
                // picard_relax_visc in log space; log of the current viscosity carried between iterations
                const R lc = have_log ? lv[ck] : log((R)vcur[ck]);
                const R L = (R(1) - rel) * lc + rel * log(v);
                vr = exp(L);
                lv[ck] = L;
            } else {
                vr = v;
                if (!visc_only) lv[ck] = log(vr);
            }
            vn[ck] = (VD)vr;
            // trapezoid integrals (integrate_trapezoid1D_pt, yelmo_tools.f90:1092-1122),
            // in the viscosity arithmetic R
            const R omz = zt.omz(k);
            const R g = (Hr / vr) * (omz * omz);
            if (k > 0) {
                const R dzt = zt.dz(k);
                vint = vint + R(0.5) * (vr + vprev) * dzt;
                f2 = f2 + R(0.5) * (g + gprev) * dzt;
            }
            vprev = vr;
            gprev = g;
        }
        if (visc_only) continue;
        // calc_visc_eff_int, velocity_general.f90:2215-2261
        double vi = ice ? (double)vint * Hc : VISC_MIN;
        if (vi < VISC_MIN) vi = VISC_MIN;
        I.visc_int[c] = vi;
        if (I.fN) I.fN[c] = (float)vi;     // mixed mode: the FP32 copy of the inner solves
        // calc_F_integral (n = 2), velocity_diva.f90:824-869
        if (diva) I.F2[c] = ice ? (double)f2 : 0.0;
        // calc_beta: SSA uses the iterate, DIVA the basal velocity
        if (P.beta_method != -1) {
            const double* ubx = diva ? I.ux_b : I.u_x;
            const double* uby = diva ? I.uy_b : I.u_y;
            I.beta[c] = beta_aa(I, P, G, n.i, n.j, ubx, uby);
        }
    }
}

// ---------------------------------------------------------------------------
// Phase: faces -- staggering, beta_eff, beta_min, drag, N_ab, drag coefficients
// ---------------------------------------------------------------------------
YG_DEV double gl_flux_weight(double beta_a, double ux_a, double ux_b, double H_a, double H_b, double f_ac) {
    // calc_beta_gl_flux_weight, basal_dragging.f90:1760-1845
    double q_a = ux_a * H_a, q_b = ux_b * H_b, ug = 0.0, ut = 0.0;
    for (int n = 1; n <= 100; n++) {
        double lam = ((double)n - 0.5) / 100.0;
        double Hn = H_a * lam + H_b * (1.0 - lam);
        double qn = q_a * lam + q_b * (1.0 - lam);
        double un = (Hn > 0.0) ? qn / Hn : 0.0;
        ut = ut + fabs(un);
        if (lam > (1.0 - f_ac)) ug = ug + fabs(un);
    }
    double w = (ut > 0.0) ? ug / ut : 0.0;
    return beta_a * w;
}

// stagger_beta for one face (basal_dragging.f90:581-704 and :1360-1758), before the limit
YG_DEV double stagger_beta_face(const Inst& I, const ygpu_dyn_par& P, const Geo& G, int i, int j, bool xdir) {
    int im1, ip1, jm1, jp1;
    nbr_bc(i, j, G.nx, G.ny, G.bc, im1, ip1, jm1, jp1);
    const int c = CI(i, j), cn = xdir ? CI(ip1, j) : CI(i, jp1);
    // the f_ice and f_grnd tests from the cell flags (the same compares, made
    // once by the setup step)
    const unsigned fc = I.cflag[c], fn = I.cflag[cn];
    const bool ice_c = (fc & CF_ICE) != 0, ice_n = (fn & CF_ICE) != 0;
    const bool part_c = (fc & CF_PART) != 0, part_n = (fn & CF_PART) != 0;
    const bool g0_c = (fc & CF_G0) != 0, g0_n = (fn & CF_G0) != 0;
    const double* be = I.beta;
    double b;
    if (g0_c && g0_n) b = 0.0;
    else if (ice_c && part_n) b = be[c];
    else if (part_c && ice_n) b = be[cn];
    else b = 0.5 * (be[c] + be[cn]);
    const int gs = P.beta_gl_stag;
    if (gs >= 1 && gs <= 4 && ice_c && ice_n) {
        const bool gl_r = ((fc & CF_GPOS) != 0) && g0_n;
        const bool gl_l = g0_c && ((fn & CF_GPOS) != 0);
        if (gs == 1) {
            if (gl_r) b = be[c]; else if (gl_l) b = be[cn];
        } else if (gs == 2) {
            if (gl_r) b = be[cn]; else if (gl_l) b = be[c];
        } else if (gs == 3) {
            double fgf = xdir ? I.fg_x[c] : I.fg_y[c];
            double wt = fgf * fgf;
            if (gl_r) b = wt * be[c] + (1.0 - wt) * be[cn];
            else if (gl_l) b = (1.0 - wt) * be[c] + wt * be[cn];
        } else {
            const double* u = xdir ? I.u_x : I.u_y;
            const int cm = xdir ? CI(im1, j) : CI(i, jm1);
            double fgf = xdir ? I.fg_x[c] : I.fg_y[c];
            if (gl_r) {
                double ua = 0.5 * (u[cm] + u[c]), ub = 0.5 * (u[cn] + u[c]);
                b = gl_flux_weight(be[c], ua, ub, I.H[c], I.H[cn], fgf);
            } else if (gl_l) {
                double ua = 0.5 * (u[cn] + u[c]), ub = 0.5 * (u[cm] + u[c]);
                b = gl_flux_weight(be[cn], ua, ub, I.H[cn], I.H[c], fgf);
            }
        }
    }
    return b;
}

// s0sq_lo: a bound below s0^2 (s0^2 (1 - 2^-40), rounded), so that a speed
// square under it has sqrt(.) <= s0 and skips the FP64 square root
YG_DEV void lim_face(double& k, double& r, double u, double uc, int mask, double s0, double s0sq_lo, double inv_du,
                     double tau_c) {
    // calc_vel_lim_drag / lim_drag_face, solver_ssa_ac.f90:1095-1199
    k = 0.0;
    r = 0.0;
    if (mask < 1) return;
    const double a = u * u + uc * uc;
    if (a <= s0sq_lo) return;
    double s = sqrt(a);
    if (s <= s0) return;
    double x = (s - s0) * inv_du;
    double tau = tau_c * x * x;
    double dtds = 2.0 * tau_c * x * inv_du;
    double b = tau / s;
    double w = (u / s) * (u / s);
    k = b * (1.0 - w) + dtds * w;
    r = (k - b) * u;
}

// R: arithmetic of the effective friction, the operator drag and N_ab: FP64 in
// the FP64 solve; FP32 in the mixed one, whose FP64 outer residual then uses
// the FP32-rounded coefficients (the same values as its FP32 inner operator)
template <typename R>
__device__ __noinline__ void phase_faces(const Inst& I, const ygpu_dyn_par& P, const Geo& Gr, Team& T, bool diva) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const Geo G = Gr;
    const int tid = t_tid, nthr = t_nthr;
    const bool energy = (P.ssa_solver == YGPU_SSA_ENERGY);
    const bool drag = (P.ssa_vel_lim_method == YGPU_VEL_LIM_DRAG);
    const bool limit = (P.beta_method != -1 && P.beta_gl_stag != -1);
    const double s0 = 0.8 * P.ssa_vel_max;
    const double s0sq_lo = (s0 * s0) * (1.0 - 0x1p-40);
    const double inv_du = 1.0 / (P.ssa_vel_max - s0);
    const int nx = G.nx, ny = G.ny;
    for (int c = tid; c < G.n2; c += nthr) {
        Nb n = make_nb(G, c);
        const int i = n.i, j = n.j;
        // staggered F2 (stagger_F_integral, velocity_diva.f90:871-910)
        double F2x = 0.0, F2y = 0.0;
        if (diva) {
            const unsigned fc = I.cflag[c];
            F2x = stag_margin_fl(I.F2[c], I.F2[CI(n.ip1, j)], fc, (unsigned)I.cflag[CI(n.ip1, j)]);
            F2y = stag_margin_fl(I.F2[c], I.F2[CI(i, n.jp1)], fc, (unsigned)I.cflag[CI(i, n.jp1)]);
            I.F2x[c] = F2x;
            I.F2y[c] = F2y;
        }
        // stagger_beta with the border copies of infinite/MISMIP3D/mask
        double bx = I.beta_x[c], by = I.beta_y[c];
        if (P.beta_gl_stag != -1) {
            int sxi = i, sxj = j, syi = i, syj = j;
            if (G.bc == YGPU_BND_INFINITE || G.bc == YGPU_BND_MISMIP3D) {
                if (i == 0) sxi = 1;
                else if (i == nx - 2 || i == nx - 1) sxi = nx - 3;
                if (i == 0) syi = 1;
                else if (i == nx - 1) syi = nx - 2;
            }
            if (G.bc == YGPU_BND_INFINITE) {
                if (j == 0) sxj = 1;
                else if (j == ny - 1) sxj = ny - 2;
                if (j == 0) syj = 1;
                else if (j == ny - 2 || j == ny - 1) syj = ny - 3;
            }
            bx = stagger_beta_face(I, P, G, sxi, sxj, true);
            by = stagger_beta_face(I, P, G, syi, syj, false);
        }
        if (limit) {
            if (bx > 0.0 && bx < P.beta_min) bx = P.beta_min;
            if (by > 0.0 && by < P.beta_min) by = P.beta_min;
        }
        I.beta_x[c] = bx;
        I.beta_y[c] = by;
        // friction used by the matrix
        R mx_b = (R)bx, my_b = (R)by;
        if (diva) {
            // calc_beta_eff, velocity_diva.f90:912-958
            const R f2x = (R)F2x, f2y = (R)F2y, f2 = (R)I.F2[c], be = (R)I.beta[c];
            if (P.no_slip) {
                mx_b = (f2x > R(0)) ? R(1) / f2x : R(0);
                my_b = (f2y > R(0)) ? R(1) / f2y : R(0);
                I.beta_eff[c] = (double)((f2 > R(0)) ? R(1) / f2 : R(0));
            } else {
                mx_b = mx_b / (R(1) + mx_b * f2x);
                my_b = my_b / (R(1) + my_b * f2y);
                I.beta_eff[c] = (double)(be / (R(1) + be * f2));
            }
        }
        // set_beta_min_grounded, basal_dragging.f90:706-780
        const int mx = I.mask_x[c], my = I.mask_y[c];
        if (mx == 1 && mx_b == R(0)) mx_b = (R)P.beta_min;
        if (my == 1 && my_b == R(0)) my_b = (R)P.beta_min;
        I.bm_x[c] = (double)mx_b;
        I.bm_y[c] = (double)my_b;
        // speed-limit drag around the iterate
        double kx = 0.0, ky = 0.0, rx = 0.0, ry = 0.0;
        if (drag) {
            const double* ux = I.u_x;
            const double* uy = I.u_y;
            double uc = 0.25 * (uy[c] + uy[CI(n.ip1, j)] + uy[CI(i, n.jm1)] + uy[CI(n.ip1, n.jm1)]);
            lim_face(kx, rx, ux[c], uc, mx, s0, s0sq_lo, inv_du, P.ssa_vel_lim_tau);
            uc = 0.25 * (ux[c] + ux[CI(n.im1, j)] + ux[CI(i, n.jp1)] + ux[CI(n.im1, n.jp1)]);
            lim_face(ky, ry, uy[c], uc, my, s0, s0sq_lo, inv_du, P.ssa_vel_lim_tau);
        }
        // the drag's right-hand-side terms (read by the system phase only with the
        // drag on); kx, ky enter the operator coefficients below
        if (drag) { I.lr_x[c] = rx; I.lr_y[c] = ry; }
        // operator drag coefficients: w*(beta + k) (* dx*dy for the energy form)
        R wx, wy, dgx, dgy;
        if (energy) {
            wx = (mx == 3 || mx == 4) ? R(0.5) : R(1);
            wy = (my == 3 || my == 4) ? R(0.5) : R(1);
            dgx = wx * (mx_b + (R)kx) * (R)G.dxdy;
            dgy = wy * (my_b + (R)ky) * (R)G.dxdy;
        } else {
            wx = (mx == 4) ? R(0.5) : R(1);
            wy = (my == 4) ? R(0.5) : R(1);
            dgx = wx * mx_b + wx * (R)kx;
            dgy = wy * my_b + wy * (R)ky;
        }
        I.drag_x[c] = (double)dgx;
        I.drag_y[c] = (double)dgy;
        if (I.fdrag_x) {               // mixed mode: FP32 copies of the inner solves
            I.fdrag_x[c] = (float)dgx;
            I.fdrag_y[c] = (float)dgy;
        }
        // stagger_visc_aa_ab, solver_ssa_ac.f90:1000-1067
        {
            const int cc[4] = {c, CI(n.ip1, j), CI(i, n.jp1), CI(n.ip1, n.jp1)};
            int nice = 0;
            bool anyocn = false;
            R v[4];
#pragma unroll
            for (int q = 0; q < 4; q++) {
                const unsigned fq = I.cflag[cc[q]];
                bool ice = (fq & CF_ICE) != 0;
                bool ocn = (fq & CF_OCN) != 0;
                nice += ice;
                anyocn = anyocn || ocn;
                v[q] = ice ? (R)I.visc_int[cc[q]] : R(0);
            }
            // the mean: a division only for three iced corners (halving and
            // quartering are exact multiplications)
            const R sum = (v[0] + v[1]) + (v[2] + v[3]);
            R nab;
            if (anyocn || nice == 0) nab = R(0);
            else if (nice == 3) nab = sum / R(3);
            else nab = sum * ((nice == 4) ? R(0.25) : (nice == 2) ? R(0.5) : R(1));
            I.Nab[c] = (double)nab;
            if (I.fNab) I.fNab[c] = (float)nab;
        }
    }
}

// ---------------------------------------------------------------------------
// Energy operator (solver_ssa_ac_energy.f90:70-708, matrix-free)
// ---------------------------------------------------------------------------
YG_DEV bool wrap_index(int& k, int nk, bool periodic, bool free_lo, bool free_hi) {
    if (k < 0) {
        if (periodic) k += nk;
        else if (free_lo) k = 0;
        else return false;
    } else if (k > nk - 1) {
        if (periodic) k -= nk;
        else if (free_hi) k = nk - 1;
        else return false;
    }
    return true;
}
YG_DEV bool elem_index(int& k, int nk, bool periodic) {
    if (k < 0 || k > nk - 1) {
        if (!periodic) return false;
        k = ((k % nk) + nk) % nk;
    }
    return true;
}
// unknown of ux(ii,jj) / uy(ii,jj) one beyond the domain allowed; -1 = zero ghost
YG_DEV int dof_u(const Geo& G, int ii, int jj, int plane) {
    if (!wrap_index(ii, G.nx, G.per_x, bfree(G.bb, 2), bfree(G.bb, 0))) return -1;
    if (!wrap_index(jj, G.ny, G.per_y, bfree(G.bb, 3), bfree(G.bb, 1))) return -1;
    return ii + G.nx * jj + plane * G.n2;
}

// Contribution of member unknown mm (plane pl, cell (i,j)) of the elements
// around it: sum over the slots holding mm of H(l,:) . val(dofs). val(d) must
// return 0 for d < 0.
template <typename T, typename CT, typename V>
YG_DEV T member_elems(const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab, int mm, V val) {
    const int pl = (mm >= G.n2) ? 1 : 0;
    const int c = mm - pl * G.n2;
    const int i = c % G.nx, j = c / G.nx;
    const T dyodx = K.dyodx, dxody = K.dxody;
    T acc = T(0);
    // cells: ux -> (i,j),(i+1,j); uy -> (i,j),(i,j+1)
#pragma unroll
    for (int e = 0; e < 2; e++) {
        int ci = (pl == 0) ? i + e : i, cj = (pl == 0) ? j : j + e;
        if (!elem_index(ci, G.nx, G.per_x) || !elem_index(cj, G.ny, G.per_y)) continue;
        int d0 = dof_u(G, ci - 1, cj, 0), d1 = dof_u(G, ci, cj, 0);
        int d2 = dof_u(G, ci, cj - 1, 1), d3 = dof_u(G, ci, cj, 1);
        if (d0 != mm && d1 != mm && d2 != mm && d3 != mm) continue;
        T Nc = (T)N[ci + G.nx * cj];
        T hx = T(4) * Nc * dyodx, hy = T(4) * Nc * dxody, hc = T(2) * Nc;
        T ex = val(d1) - val(d0), ey = val(d3) - val(d2);
        T Fx = hx * ex + hc * ey, Fy = hc * ex + hy * ey;
        if (d0 == mm) acc -= Fx;
        if (d1 == mm) acc += Fx;
        if (d2 == mm) acc -= Fy;
        if (d3 == mm) acc += Fy;
    }
    // corners: ux -> (i,j),(i,j-1); uy -> (i,j),(i-1,j)
#pragma unroll
    for (int e = 0; e < 2; e++) {
        int ci = (pl == 0) ? i : i - e, cj = (pl == 0) ? j - e : j;
        if (!elem_index(ci, G.nx, G.per_x) || !elem_index(cj, G.ny, G.per_y)) continue;
        int d0 = dof_u(G, ci, cj, 0), d1 = dof_u(G, ci, cj + 1, 0);
        int d2 = dof_u(G, ci, cj, 1), d3 = dof_u(G, ci + 1, cj, 1);
        if (d0 != mm && d1 != mm && d2 != mm && d3 != mm) continue;
        T Nc = (T)Nab[ci + G.nx * cj];
        T sx = val(d1) - val(d0), sy = val(d3) - val(d2);
        T G1 = Nc * (dxody * sx + sy), G2 = Nc * (sx + dyodx * sy);
        if (d0 == mm) acc -= G1;
        if (d1 == mm) acc += G1;
        if (d2 == mm) acc -= G2;
        if (d3 == mm) acc += G2;
    }
    return acc;
}

// Interior fast path: a free row whose 4 elements hold only free, self-mapped
// unknowns (no Dirichlet, tied or ghost columns) is the 9-point stencil
// K = -A_residual * dx*dy (the identity the reference's test_ssa_energy pins).
template <typename T, typename CT>
YG_DEV T energy_row_fast(const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab, const CT* dgx, const CT* dgy,
                         const T* v, int u) {
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    const int pl = (u >= n2) ? 1 : 0;
    const int c = u - pl * n2;
    const int i = c % nx, j = c / nx;
    const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
    const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
    const T dyodx = K.dyodx, dxody = K.dxody;
    const T* U = v;
    const T* V = v + n2;
    if (pl == 0) {
        const T Ni = (T)N[c], Np = (T)N[ip1 + nx * j];
        const T Bc = (T)Nab[c], Bm = (T)Nab[i + nx * jm1];
        T y = (T(4) * dyodx * (Np + Ni) + dxody * (Bc + Bm) + (T)dgx[c]) * U[c];
        y -= T(4) * dyodx * Np * U[ip1 + nx * j];
        y -= T(4) * dyodx * Ni * U[im1 + nx * j];
        y -= dxody * Bc * U[i + nx * jp1];
        y -= dxody * Bm * U[i + nx * jm1];
        y += (T(2) * Ni + Bc) * V[c];
        y -= (T(2) * Np + Bc) * V[ip1 + nx * j];
        y += (T(2) * Np + Bm) * V[ip1 + nx * jm1];
        y -= (T(2) * Ni + Bm) * V[i + nx * jm1];
        return y;
    } else {
        const T Ni = (T)N[c], Np = (T)N[i + nx * jp1];
        const T Bc = (T)Nab[c], Bm = (T)Nab[im1 + nx * j];
        T y = (T(4) * dxody * (Np + Ni) + dyodx * (Bc + Bm) + (T)dgy[c]) * V[c];
        y -= T(4) * dxody * Np * V[i + nx * jp1];
        y -= T(4) * dxody * Ni * V[i + nx * jm1];
        y -= dyodx * Bc * V[ip1 + nx * j];
        y -= dyodx * Bm * V[im1 + nx * j];
        y += (T(2) * Ni + Bc) * U[c];
        y -= (T(2) * Np + Bc) * U[i + nx * jp1];
        y += (T(2) * Np + Bm) * U[im1 + nx * jp1];
        y -= (T(2) * Ni + Bm) * U[im1 + nx * j];
        return y;
    }
}

// Both rows of cell c = (i, j) on the interior stencil (the two rows of
// energy_row_fast with the same arithmetic, sharing the index math and the
// loads of N, N_ab and the velocities both rows read).
template <typename T, typename CT>
YG_DEV void energy_cell_fast(const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab, const CT* dgx, const CT* dgy,
                             const T* v, int c, int i, int j, T& yx, T& yy) {
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
    const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
    const T dyodx = K.dyodx, dxody = K.dxody;
    const T* U = v;
    const T* V = v + n2;
    const int c_ip1 = ip1 + nx * j, c_im1 = im1 + nx * j, c_jp1 = i + nx * jp1, c_jm1 = i + nx * jm1;
    const T Ni = (T)N[c], Npx = (T)N[c_ip1], Npy = (T)N[c_jp1];
    const T Bc = (T)Nab[c], Bmx = (T)Nab[c_jm1], Bmy = (T)Nab[c_im1];
    const T Uc = U[c], Vc = V[c];
    const T U_ip1 = U[c_ip1], U_im1 = U[c_im1], U_jp1 = U[c_jp1], U_jm1 = U[c_jm1], U_im1jp1 = U[im1 + nx * jp1];
    const T V_ip1 = V[c_ip1], V_im1 = V[c_im1], V_jp1 = V[c_jp1], V_jm1 = V[c_jm1], V_ip1jm1 = V[ip1 + nx * jm1];
    {
        const T Np = Npx, Bm = Bmx;
        T y = (T(4) * dyodx * (Np + Ni) + dxody * (Bc + Bm) + (T)dgx[c]) * Uc;
        y -= T(4) * dyodx * Np * U_ip1;
        y -= T(4) * dyodx * Ni * U_im1;
        y -= dxody * Bc * U_jp1;
        y -= dxody * Bm * U_jm1;
        y += (T(2) * Ni + Bc) * Vc;
        y -= (T(2) * Np + Bc) * V_ip1;
        y += (T(2) * Np + Bm) * V_ip1jm1;
        y -= (T(2) * Ni + Bm) * V_jm1;
        yx = y;
    }
    {
        const T Np = Npy, Bm = Bmy;
        T y = (T(4) * dxody * (Np + Ni) + dyodx * (Bc + Bm) + (T)dgy[c]) * Vc;
        y -= T(4) * dxody * Np * V_jp1;
        y -= T(4) * dxody * Ni * V_jm1;
        y -= dyodx * Bc * V_ip1;
        y -= dyodx * Bm * V_im1;
        y += (T(2) * Ni + Bc) * Uc;
        y -= (T(2) * Np + Bc) * U_jp1;
        y += (T(2) * Np + Bm) * U_im1jp1;
        y -= (T(2) * Ni + Bm) * U_im1;
        yy = y;
    }
}

template <typename T, typename CT>
__device__ __noinline__ T energy_row_general(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N,
                                             const CT* Nab, const CT* dgx, const CT* dgy, const T* v, int u);

// Row u of K v (identity on Dirichlet and tied rows)
template <typename T, typename CT>
YG_DEV T energy_row(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab, const CT* dgx,
                    const CT* dgy, const T* v, int u) {
    // the interior stencil is evaluated for every row (its neighbour indices are
    // always in range), so its loads do not wait on the row-kind load
    const T yf = energy_row_fast<T, CT>(G, K, N, Nab, dgx, dgy, v, u);
    if (I.rpart[u] == 1) return yf;
    return energy_row_general<T, CT>(I, G, K, N, Nab, dgx, dgy, v, u);
}

// Row u of K v outside the interior stencil: Dirichlet and tied rows are the
// identity; free rows sum the element derivatives of the unknown and of the
// unknowns tied to it
template <typename T, typename CT>
__device__ __noinline__ T energy_row_general(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N,
                                             const CT* Nab, const CT* dgx, const CT* dgy, const T* v, int u) {
    if (I.ukind[u] != DOF_FREE) return v[u];
    const int* emap = I.emap;
    auto val = [&](int d) -> T {
        if (d < 0) return T(0);
        int e = emap[d];
        return (e >= 0) ? v[e] : T(0);
    };
    const T vr = v[u];
    T acc = ((u < G.n2) ? (T)dgx[u] : (T)dgy[u - G.n2]) * vr;
    acc += member_elems<T>(G, K, N, Nab, u, val);
    const int* mem = I.mem + 3 * u;
    for (int m = 0; m < 3; m++) {
        int mm = mem[m];
        if (mm < 0) break;
        acc += ((mm < G.n2) ? (T)dgx[mm] : (T)dgy[mm - G.n2]) * vr;
        acc += member_elems<T>(G, K, N, Nab, mm, val);
    }
    return acc;
}

// ---------------------------------------------------------------------------
// Residual operator (solver_ssa_ac.f90:73-848, matrix-free)
// ---------------------------------------------------------------------------
template <typename T, typename CT>
YG_DEV T residual_row(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab, const CT* dgx,
                      const CT* dgy, const T* v, int u, T* diag_out) {
    const int rk = I.ukind[u];
    if (rk == RROW_ID) {
        if (diag_out) *diag_out = T(1);
        return v[u];
    }
    if (rk == RROW_FREESLIP) {
        if (diag_out) *diag_out = T(1);
        return v[u] - v[I.rpart[u]];
    }
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    const int pl = (u >= n2) ? 1 : 0;
    const int c = u - pl * n2;
    const int i = c % nx, j = c / nx;
    const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
    const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
    const T inv_dx = K.inv_dx, inv_dy = K.inv_dy;
    const T inv_dxdx = K.inv_dxdx, inv_dydy = K.inv_dydy, inv_dxdy = K.inv_dxdy;
#define VX(a, b) v[(a) + nx * (b)]
#define VY(a, b) v[n2 + (a) + nx * (b)]
#define NN(a, b) ((T)N[(a) + nx * (b)])
#define NB(a, b) ((T)Nab[(a) + nx * (b)])
    if (rk == RROW_FRONT) {
        if (pl == 0) {
            if (I.f_ice[c] == 1.0 && I.f_ice[ip1 + nx * j] < 1.0) {
                T Nn = NN(i, j);
                if (diag_out) *diag_out = T(4) * inv_dx * Nn;
                return -T(4) * inv_dx * Nn * VX(im1, j) - T(2) * inv_dy * Nn * VY(i, jm1) + T(4) * inv_dx * Nn * VX(i, j) +
                       T(2) * inv_dy * Nn * VY(i, j);
            }
            T Nn = NN(ip1, j);
            if (diag_out) *diag_out = -T(4) * inv_dx * Nn;
            return -T(4) * inv_dx * Nn * VX(i, j) - T(2) * inv_dy * Nn * VY(ip1, jm1) + T(4) * inv_dx * Nn * VX(ip1, j) +
                   T(2) * inv_dy * Nn * VY(ip1, j);
        } else {
            if (I.f_ice[c] == 1.0 && I.f_ice[i + nx * jp1] < 1.0) {
                T Nn = NN(i, j);
                if (diag_out) *diag_out = T(4) * inv_dy * Nn;
                return -T(2) * inv_dx * Nn * VX(im1, j) - T(4) * inv_dy * Nn * VY(i, jm1) + T(2) * inv_dx * Nn * VX(i, j) +
                       T(4) * inv_dy * Nn * VY(i, j);
            }
            T Nn = NN(i, jp1);
            if (diag_out) *diag_out = -T(4) * inv_dy * Nn;
            return -T(2) * inv_dx * Nn * VX(im1, jp1) - T(4) * inv_dy * Nn * VY(i, j) + T(2) * inv_dx * Nn * VX(i, jp1) +
                   T(4) * inv_dy * Nn * VY(i, jp1);
        }
    }
    // inner SSA rows
    if (pl == 0) {
        T d = -T(4) * inv_dxdx * (NN(ip1, j) + NN(i, j)) - T(1) * inv_dydy * (NB(i, j) + NB(i, jm1)) - (T)dgx[c];
        if (diag_out) *diag_out = d;
        T s = d * VX(i, j);
        s += T(4) * inv_dxdx * NN(ip1, j) * VX(ip1, j);
        s += T(4) * inv_dxdx * NN(i, j) * VX(im1, j);
        s += T(1) * inv_dydy * NB(i, j) * VX(i, jp1);
        s += T(1) * inv_dydy * NB(i, jm1) * VX(i, jm1);
        s += (-T(2) * inv_dxdy * NN(i, j) - T(1) * inv_dxdy * NB(i, j)) * VY(i, j);
        s += (T(2) * inv_dxdy * NN(ip1, j) + T(1) * inv_dxdy * NB(i, j)) * VY(ip1, j);
        s += (-T(2) * inv_dxdy * NN(ip1, j) - T(1) * inv_dxdy * NB(i, jm1)) * VY(ip1, jm1);
        s += (T(2) * inv_dxdy * NN(i, j) + T(1) * inv_dxdy * NB(i, jm1)) * VY(i, jm1);
        return s;
    } else {
        T d = -T(4) * inv_dydy * (NN(i, jp1) + NN(i, j)) - T(1) * inv_dxdx * (NB(i, j) + NB(im1, j)) - (T)dgy[c];
        if (diag_out) *diag_out = d;
        T s = d * VY(i, j);
        s += T(4) * inv_dydy * NN(i, jp1) * VY(i, jp1);
        s += T(4) * inv_dydy * NN(i, j) * VY(i, jm1);
        s += T(1) * inv_dxdx * NB(i, j) * VY(ip1, j);
        s += T(1) * inv_dxdx * NB(im1, j) * VY(im1, j);
        s += (-T(2) * inv_dxdy * NN(i, j) - T(1) * inv_dxdy * NB(i, j)) * VX(i, j);
        s += (T(2) * inv_dxdy * NN(i, jp1) + T(1) * inv_dxdy * NB(i, j)) * VX(i, jp1);
        s += (-T(2) * inv_dxdy * NN(i, jp1) - T(1) * inv_dxdy * NB(im1, j)) * VX(im1, jp1);
        s += (T(2) * inv_dxdy * NN(i, j) + T(1) * inv_dxdy * NB(im1, j)) * VX(im1, j);
        return s;
    }
#undef VX
#undef VY
#undef NN
#undef NB
}

// ---------------------------------------------------------------------------
// ILU(0) of the residual form (-p ilu with BiCGSTAB, solver_linear.F90:246-395
// hands "-p ilu" to LIS). The factorization is ILU(0) (Saad, Iterative Methods,
// 10.3: no fill outside the pattern of A) of A in a six-colour ordering: cell
// colour (i - j) mod 3 and then the component, ux before uy. No two coupled
// unknowns share a colour group (neighbours differ in cell colour; the two
// components of a cell are in different groups), so the rows of a group factor
// and solve independently; a thread takes both rows of a cell, whose only
// coupling inside their colour is to each other, so a team barrier separates the
// three cell colours: 3 barriers for the factorization, 3 + 3 for an
// application. Rows are YG_ILU_W slots in a fixed stencil layout; a slot's
// column carries its group in bits 28..30.
// ---------------------------------------------------------------------------
// the colouring needs the periodic directions in multiples of 3 (Jacobi otherwise)
YG_DEV bool ilu_colourable(const Geo& G) {
    bool px, py;
    periodic_dirs(G.bc, px, py);
    return !(px && G.nx % 3 != 0) && !(py && G.ny % 3 != 0);
}
YG_DEV int ilu_group(int nx, int n2, int u) {
    const int pl = (u >= n2) ? 1 : 0;
    const int c = u - pl * n2;
    const int i = c % nx, j = c / nx;
    return 2 * (((i - j) % 3 + 3) % 3) + pl;
}
// The cells of colour gc, (i - j) mod 3 == gc, for a team of nthr threads.
// With fewer threads than cells (batches), slot t = j * m + k holds cell
// (i0(j) + 3 k, j), i0(j) = (j + gc) mod 3, m = ceil(nx / 3): no slot of another
// colour, so every lane of a warp works. With a thread per cell (small single
// solves) slot t is cell t, and the cells of other colours are skipped: their
// lanes idle, but the colour's rows spread over three times as many warps,
// which hides the FP64 latency of a row's elimination better (measured).
// Returns -1 for a slot without a cell of colour gc.
struct IluColour {
    int nx, n2, m, slots;
    bool compact;
    YG_DEV IluColour(int nx_, int n2_, int nthr) : nx(nx_), n2(n2_) {
        m = (nx + 2) / 3;
        compact = nthr < n2;
        slots = compact ? (n2 / nx) * m : n2;
    }
    YG_DEV int cell(int gc, int t) const {
        if (!compact) {
            const int j = t / nx, i = t - j * nx;
            return (((i - j) % 3 + 3) % 3 == gc) ? t : -1;
        }
        const int j = t / m;
        const int i = (j + gc) % 3 + 3 * (t - j * m);
        return (i < nx) ? i + nx * j : -1;
    }
};
// The coefficients of residual_row (same formulas) for row u: col[s] = -1 for
// unused slots. Slots: 0 the diagonal, then the row's stencil in the order of
// residual_row.
template <typename T, typename CT>
YG_DEV void residual_row_coefs(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N, const CT* Nab,
                               const CT* dgx, const CT* dgy, int u, int col[YG_ILU_W], T val[YG_ILU_W]) {
#pragma unroll
    for (int s = 0; s < YG_ILU_W; s++) { col[s] = -1; val[s] = T(0); }
    col[0] = u;
    const int rk = I.ukind[u];
    if (rk == RROW_ID) { val[0] = T(1); return; }
    if (rk == RROW_FREESLIP) {
        val[0] = T(1);
        col[1] = I.rpart[u];
        val[1] = T(-1);
        return;
    }
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    const int pl = (u >= n2) ? 1 : 0;
    const int c = u - pl * n2;
    const int i = c % nx, j = c / nx;
    const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
    const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
    const T inv_dx = K.inv_dx, inv_dy = K.inv_dy;
    const T inv_dxdx = K.inv_dxdx, inv_dydy = K.inv_dydy, inv_dxdy = K.inv_dxdy;
    auto X = [&](int a, int b) { return a + nx * b; };
    auto Y = [&](int a, int b) { return n2 + a + nx * b; };
    auto NN = [&](int a, int b) { return (T)N[a + nx * b]; };
    auto NB = [&](int a, int b) { return (T)Nab[a + nx * b]; };
    if (rk == RROW_FRONT) {
        if (pl == 0) {
            if (I.f_ice[c] == 1.0 && I.f_ice[ip1 + nx * j] < 1.0) {
                const T Nn = NN(i, j);
                val[0] = T(4) * inv_dx * Nn;
                col[1] = X(im1, j); val[1] = -T(4) * inv_dx * Nn;
                col[2] = Y(i, jm1); val[2] = -T(2) * inv_dy * Nn;
                col[3] = Y(i, j); val[3] = T(2) * inv_dy * Nn;
            } else {
                const T Nn = NN(ip1, j);
                val[0] = -T(4) * inv_dx * Nn;
                col[1] = Y(ip1, jm1); val[1] = -T(2) * inv_dy * Nn;
                col[2] = X(ip1, j); val[2] = T(4) * inv_dx * Nn;
                col[3] = Y(ip1, j); val[3] = T(2) * inv_dy * Nn;
            }
        } else {
            if (I.f_ice[c] == 1.0 && I.f_ice[i + nx * jp1] < 1.0) {
                const T Nn = NN(i, j);
                val[0] = T(4) * inv_dy * Nn;
                col[1] = X(im1, j); val[1] = -T(2) * inv_dx * Nn;
                col[2] = Y(i, jm1); val[2] = -T(4) * inv_dy * Nn;
                col[3] = X(i, j); val[3] = T(2) * inv_dx * Nn;
            } else {
                const T Nn = NN(i, jp1);
                val[0] = -T(4) * inv_dy * Nn;
                col[1] = X(im1, jp1); val[1] = -T(2) * inv_dx * Nn;
                col[2] = X(i, jp1); val[2] = T(2) * inv_dx * Nn;
                col[3] = Y(i, jp1); val[3] = T(4) * inv_dy * Nn;
            }
        }
    } else if (pl == 0) {
        val[0] = -T(4) * inv_dxdx * (NN(ip1, j) + NN(i, j)) - T(1) * inv_dydy * (NB(i, j) + NB(i, jm1)) - (T)dgx[c];
        col[1] = X(ip1, j); val[1] = T(4) * inv_dxdx * NN(ip1, j);
        col[2] = X(im1, j); val[2] = T(4) * inv_dxdx * NN(i, j);
        col[3] = X(i, jp1); val[3] = T(1) * inv_dydy * NB(i, j);
        col[4] = X(i, jm1); val[4] = T(1) * inv_dydy * NB(i, jm1);
        col[5] = Y(i, j); val[5] = -T(2) * inv_dxdy * NN(i, j) - T(1) * inv_dxdy * NB(i, j);
        col[6] = Y(ip1, j); val[6] = T(2) * inv_dxdy * NN(ip1, j) + T(1) * inv_dxdy * NB(i, j);
        col[7] = Y(ip1, jm1); val[7] = -T(2) * inv_dxdy * NN(ip1, j) - T(1) * inv_dxdy * NB(i, jm1);
        col[8] = Y(i, jm1); val[8] = T(2) * inv_dxdy * NN(i, j) + T(1) * inv_dxdy * NB(i, jm1);
    } else {
        val[0] = -T(4) * inv_dydy * (NN(i, jp1) + NN(i, j)) - T(1) * inv_dxdx * (NB(i, j) + NB(im1, j)) - (T)dgy[c];
        col[1] = Y(i, jp1); val[1] = T(4) * inv_dydy * NN(i, jp1);
        col[2] = Y(i, jm1); val[2] = T(4) * inv_dydy * NN(i, j);
        col[3] = Y(ip1, j); val[3] = T(1) * inv_dxdx * NB(i, j);
        col[4] = Y(im1, j); val[4] = T(1) * inv_dxdx * NB(im1, j);
        col[5] = X(i, j); val[5] = -T(2) * inv_dxdy * NN(i, j) - T(1) * inv_dxdy * NB(i, j);
        col[6] = X(i, jp1); val[6] = T(2) * inv_dxdy * NN(i, jp1) + T(1) * inv_dxdy * NB(i, j);
        col[7] = X(im1, jp1); val[7] = -T(2) * inv_dxdy * NN(i, jp1) - T(1) * inv_dxdy * NB(im1, j);
        col[8] = X(im1, j); val[8] = T(2) * inv_dxdy * NN(i, j) + T(1) * inv_dxdy * NB(im1, j);
    }
    // repeated columns (grids of side 2 or less) merge into their first slot
#pragma unroll
    for (int s = 1; s < YG_ILU_W; s++) {
        if (col[s] < 0) continue;
        for (int t = 0; t < s; t++)
            if (col[t] == col[s]) { val[t] += val[s]; col[s] = -1; val[s] = T(0); break; }
    }
}

// ILU(0) factors of A (coefficients N, Nab, dgx, dgy) into lu / pivinv / icol.
// Colour by colour (a team barrier after each); a thread factors both rows of a
// cell, ux (group 2 gc) then uy (group 2 gc + 1): the only column of a row in
// its own colour is the other component of the same cell, which the same
// thread has just factored. Returns false if the team is aborting.
template <typename T, typename CT>
__device__ __noinline__ bool ilu_factor(const Inst& I, const Geo& G, Team& T_, const CT* N, const CT* Nab,
                                        const CT* dgx, const CT* dgy, T* lu, T* pivinv) {
    const OpK<T> K = make_opk<T>(G);
    const int nx = G.nx, n2 = G.n2;
    const int tid = T_.tid, nthr = T_.nthr;
    int* icol = I.icol;
    const IluColour cl(nx, n2, nthr);
    for (int gc = 0; gc < 3; gc++) {
        for (int t = tid; t < cl.slots; t += nthr) {
            const int c = cl.cell(gc, t);
            if (c < 0) continue;
#pragma unroll 1
            for (int h = 0; h < 2; h++) {
                const int u = c + h * n2;
                const int g = 2 * gc + h;
                int col[YG_ILU_W];
                T a[YG_ILU_W];
                residual_row_coefs<T, CT>(I, G, K, N, Nab, dgx, dgy, u, col, a);
                int grp[YG_ILU_W];
#pragma unroll
                for (int q = 0; q < YG_ILU_W; q++) grp[q] = (col[q] >= 0) ? ilu_group(nx, n2, col[q]) : -1;
                const T d0 = a[0];
                // IKJ elimination against the factored rows before this one, in group order
                for (int gk = 0; gk < g; gk++) {
                    for (int q = 1; q < YG_ILU_W; q++) {
                        if (grp[q] != gk) continue;
                        const int k = col[q];
                        const T l = a[q] * pivinv[k];
                        a[q] = l;
                        const int* ck = icol + (size_t)k * YG_ILU_W;
                        const T* vk = lu + (size_t)k * YG_ILU_W;
                        for (int t = 1; t < YG_ILU_W; t++) {
                            const int pc = ck[t];
                            if (pc < 0 || (pc >> 28) <= gk) continue;      // the U part of row k
                            const int cj = pc & 0x0fffffff;
                            const T ukj = vk[t];
                            for (int q2 = 0; q2 < YG_ILU_W; q2++)
                                if (col[q2] == cj) { a[q2] -= l * ukj; break; }
                        }
                    }
                }
                // a pivot that cancels is replaced by the row's own diagonal (as the oracle)
                T piv = a[0];
                if (fabs((double)piv) <= 1e-14 * fabs((double)d0)) piv = d0;
                if (piv == T(0)) piv = T(1);
                a[0] = piv;
                int* cu = icol + (size_t)u * YG_ILU_W;
                T* vu = lu + (size_t)u * YG_ILU_W;
#pragma unroll
                for (int q = 0; q < YG_ILU_W; q++) {
                    cu[q] = (col[q] >= 0) ? (col[q] | (grp[q] << 28)) : -1;
                    vu[q] = a[q];
                }
                pivinv[u] = T(1) / piv;
            }
        }
        if (!team_barrier(T_)) return false;
    }
    return true;
}

// z = (LU)^-1 r over every row: forward substitution colour by colour (ux row,
// then uy row of each cell), then backward (uy row, then ux row). z may not
// alias r. Ends with a team barrier (z is read at neighbouring rows next).
template <typename T>
YG_DEV bool ilu_apply(Team& T_, int nx, int n2, int nu, const int* __restrict__ icol, const T* __restrict__ lu,
                      const T* __restrict__ pivinv, const T* r, T* z) {
    (void)nu;
    const int tid = T_.tid, nthr = T_.nthr;
    const IluColour cl(nx, n2, nthr);
    for (int gc = 0; gc < 3; gc++) {
        for (int t = tid; t < cl.slots; t += nthr) {
            const int c = cl.cell(gc, t);
            if (c < 0) continue;
#pragma unroll
            for (int h = 0; h < 2; h++) {
                const int u = c + h * n2, g = 2 * gc + h;
                const int* cu = icol + (size_t)u * YG_ILU_W;
                const T* vu = lu + (size_t)u * YG_ILU_W;
                T s = r[u];
#pragma unroll
                for (int t = 1; t < YG_ILU_W; t++) {
                    const int pc = cu[t];
                    if (pc >= 0 && (pc >> 28) < g) s -= vu[t] * z[pc & 0x0fffffff];
                }
                z[u] = s;
            }
        }
        if (!team_barrier(T_)) return false;
    }
    for (int gc = 2; gc >= 0; gc--) {
        for (int t = tid; t < cl.slots; t += nthr) {
            const int c = cl.cell(gc, t);
            if (c < 0) continue;
#pragma unroll
            for (int h = 1; h >= 0; h--) {
                const int u = c + h * n2, g = 2 * gc + h;
                const int* cu = icol + (size_t)u * YG_ILU_W;
                const T* vu = lu + (size_t)u * YG_ILU_W;
                T s = z[u];
#pragma unroll
                for (int t = 1; t < YG_ILU_W; t++) {
                    const int pc = cu[t];
                    if (pc >= 0 && (pc >> 28) > g) s -= vu[t] * z[pc & 0x0fffffff];
                }
                z[u] = s * pivinv[u];
            }
        }
        if (!team_barrier(T_)) return false;
    }
    return true;
}
template <typename T>
struct IluM {
    int nx, n2;
    const int* icol;
    const T* lu;
    const T* pivinv;
};

template <typename T, typename CT>
YG_DEV T operator_row(const Inst& I, const Geo& G, const OpK<T>& K, bool energy, const CT* N, const CT* Nab,
                      const CT* dgx, const CT* dgy, const T* v, int u) {
    if (energy) return energy_row<T, CT>(I, G, K, N, Nab, dgx, dgy, v, u);
    return residual_row<T, CT>(I, G, K, N, Nab, dgx, dgy, v, u, nullptr);
}

#define YG_ITEM_CACHE 8
#define YG_ITEM_BLOCK 512
// Per-thread work items of the Krylov loops cached in shared memory
// (thread-private slots: slot q of a thread at q * blockDim.x + threadIdx.x),
// one buffer for all the solvers of a kernel.
__shared__ int g_item_cache[YG_ITEM_CACHE * YG_ITEM_BLOCK];

// Rows a thread owns in the BiCGSTAB loops: item t is row t without an
// active-cell list, else the listed cells' ux rows then their uy rows. Each CTA
// of the team takes one contiguous chunk of the items (every SM gets rows, and
// neighbouring threads take neighbouring rows); a thread's items are t0, t0 +
// ts, ... below t1.
struct RowItems {
    const int* ac;
    int n2, nact, nitem, cache;
    int t0, t1, ts;
    YG_DEV int lookup(int t) const {
        if (!ac) return t;
        return (t < nact) ? ac[t] : n2 + ac[t - nact];
    }
    YG_DEV int row(int t, int q) const {
        return (q < cache) ? g_item_cache[q * blockDim.x + threadIdx.x] : lookup(t);
    }
};
// use_cache = false: the rows are looked up every time (for a caller whose
// items must survive calls of the solvers, which refill the cache)
YG_DEV RowItems make_row_items(const Team& Tm, const int* ac, int n2, int nu, bool use_cache = true) {
    RowItems R;
    R.ac = ac;
    R.n2 = n2;
    R.nact = ac ? min(max(ac[n2], 0), n2) : n2;
    R.nitem = ac ? 2 * R.nact : nu;
    R.cache = (use_cache && blockDim.x <= YG_ITEM_BLOCK) ? YG_ITEM_CACHE : 0;
    const int chunk = (R.nitem + Tm.ncta - 1) / Tm.ncta;
    const int beg = min(Tm.cta * chunk, R.nitem);
    R.t0 = beg + (int)threadIdx.x;
    R.t1 = min(beg + chunk, R.nitem);
    R.ts = (int)blockDim.x;
    int q = 0;
    for (int t = R.t0; t < R.t1 && q < R.cache; t += R.ts, q++)
        g_item_cache[q * blockDim.x + threadIdx.x] = R.lookup(t);
    return R;
}
template <typename Op>
YG_DEV const int* op_acell(const Op& A) { return A.acell; }

// Operator functors for the Krylov solvers: row(u, v) = (A v)_u
template <typename T, typename CT>
struct StencilOp {
    const Inst* I;
    const Geo* G;
    bool energy;
    const CT *N, *Nab, *dgx, *dgy;
    OpK<T> K;
    const int* acell = nullptr;    // active-cell list of the Krylov loops (nullptr: every cell)
    YG_DEV T row(int u, const T* v) const { return operator_row<T, CT>(*I, *G, K, energy, N, Nab, dgx, dgy, v, u); }
    YG_DEV int nx() const { return G->nx; }
    YG_DEV int n2() const { return G->n2; }
    // kind of row u in the Krylov loops of the energy form: 0 interior stencil,
    // 1 identity (Dirichlet or tied: every Krylov vector is 0 there), 2 general
    YG_DEV unsigned row_kind(int u) const {
        if (!energy) return 2u;
        if (I->rpart[u] == 1) return 0u;
        return (I->ukind[u] != DOF_FREE) ? 1u : 2u;
    }
    // row u outside the interior stencil
    YG_DEV T general(int u, const T* v) const {
        if (!energy) return residual_row<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, u, nullptr);
        return energy_row_general<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, u);
    }
    // both rows of cell c = (i, j) on the interior stencil (energy form)
    YG_DEV void cell_fast(int c, int i, int j, const T* v, T& y0, T& y1) const {
        energy_cell_fast<T, CT>(*G, K, N, Nab, dgx, dgy, v, c, i, j, y0, y1);
    }
    // both rows of cell c = (i, j): ux row c and uy row n2 + c
    YG_DEV void cell(int c, int i, int j, const T* v, T& y0, T& y1) const {
        const int n2 = G->n2;
        if (energy) {
            energy_cell_fast<T, CT>(*G, K, N, Nab, dgx, dgy, v, c, i, j, y0, y1);
            if (I->rpart[c] != 1) y0 = energy_row_general<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, c);
            if (I->rpart[n2 + c] != 1) y1 = energy_row_general<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, n2 + c);
        } else {
            y0 = residual_row<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, c, nullptr);
            y1 = residual_row<T, CT>(*I, *G, K, N, Nab, dgx, dgy, v, n2 + c, nullptr);
        }
    }
    // y = A v on the rows of R (the rows of the thread's items, as in the
    // callers' vector loops that read y right after without a barrier). FP32:
    // two rows per thread and trip, both rows' loads issued before either store.
    YG_DEV void apply(Team& Tm, const T* v, T* y, const RowItems& R) const {
        if (sizeof(T) != sizeof(float)) {
            int q = 0;
            for (int t = R.t0; t < R.t1; t += R.ts, q++) {
                const int k = R.row(t, q);
                y[k] = row(k, v);
            }
            return;
        }
        int q0 = 0;
        for (int t0 = R.t0; t0 < R.t1; t0 += 2 * R.ts, q0 += 2) {
            const int t1 = t0 + R.ts;
            const bool h1 = t1 < R.t1;
            const int k0 = R.row(t0, q0);
            const int k1 = h1 ? R.row(t1, q0 + 1) : k0;
            const T y0 = row(k0, v);
            const T y1 = row(k1, v);
            y[k0] = y0;
            if (h1) y[k1] = y1;
        }
    }
    // y = A v. Row k belongs to thread k mod nthr, as in the callers' vector
    // loops that read y right after without a barrier. FP32: two rows per
    // thread and trip, both rows' loads issued before either store.
    YG_DEV void operator()(Team& Tm, const T* v, T* y) const {
        const int nu = G->nu;
        if (sizeof(T) != sizeof(float)) {
            for (int k = Tm.tid; k < nu; k += Tm.nthr) y[k] = row(k, v);
            return;
        }
        for (int k0 = Tm.tid; k0 < nu; k0 += 2 * Tm.nthr) {
            const int k1 = k0 + Tm.nthr;
            const bool h1 = k1 < nu;
            const T y0 = row(k0, v);
            const T y1 = row(h1 ? k1 : k0, v);
            y[k0] = y0;
            if (h1) y[k1] = y1;
        }
    }
};

// CSR matrix (0-based), the lower seam linear_solver_matrix_solve
struct CsrOp {
    int n;
    const int* ptr;
    const int* idx;
    const double* val;
    const int* acell = nullptr;     // no active-cell list: every row
    YG_DEV int n2() const { return n; }
    YG_DEV void apply(Team& Tm, const double* v, double* y, const RowItems& R) const {
        int q = 0;
        for (int t = R.t0; t < R.t1; t += R.ts, q++) {
            const int k = R.row(t, q);
            y[k] = row(k, v);
        }
    }
    YG_DEV double row(int r, const double* v) const {
        double s = 0.0;
        for (int k = ptr[r]; k < ptr[r + 1]; k++) s += val[k] * v[idx[k]];
        return s;
    }
    YG_DEV void operator()(Team& Tm, const double* v, double* y) const {
        for (int r = Tm.tid; r < n; r += Tm.nthr) y[r] = row(r, v);
    }
};

// ---------------------------------------------------------------------------
// Solve setup: unknown classification (energy) or row kinds (residual)
// ---------------------------------------------------------------------------
// Active-cell list of the Krylov loops (I.acell): the cells with at least one
// non-identity row, in cell order (so the margin cells, whose rows take the
// general operator path, stay spread over the warps). Each CTA compacts a
// contiguous range of cells at the offset the CTAs before it leave, so the
// list does not depend on timing. Identity rows (Dirichlet and tied unknowns
// of the energy form, identity rows of the residual form) enter the solve with
// x = b, so their residual and Krylov vectors stay zero and the iterations
// skip the cells whose two rows are identity.
__device__ __noinline__ bool build_active_cells(const Inst& I, const Geo& G, Team& T, bool energy) {
    const int n2 = G.n2;
    auto ident = [&](int u) { return energy ? (I.ukind[u] != DOF_FREE) : (I.ukind[u] == RROW_ID); };
    auto active = [&](int c) { return !(ident(c) && ident(n2 + c)); };
    const int per = (n2 + T.ncta - 1) / T.ncta;
    const int lo = min(n2, T.cta * per), hi = min(n2, lo + per);
    __shared__ int s_cnt;
    __shared__ int s_w[32];
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    int my = 0;
    for (int c = lo + (int)threadIdx.x; c < hi; c += blockDim.x) my += active(c) ? 1 : 0;
    my = warp_sum<int>(my);
    if ((threadIdx.x & 31) == 0) atomicAdd(&s_cnt, my);
    __syncthreads();
    const double mine = (double)s_cnt;
    double before, total;
    if (!team_scan_cta(T, &mine, &before, &total, 1)) return false;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int off = (int)before;
    int bad = 0;
    for (int base = lo; base < hi; base += blockDim.x) {
        const int c = base + (int)threadIdx.x;
        const bool f = (c < hi) && active(c);
        const unsigned m = __ballot_sync(0xffffffffu, f);
        if (lane == 0) s_w[wid] = __popc(m);
        __syncthreads();
        int wbase = 0, tot = 0;
        for (int w = 0; w < nw; w++) {
            const int n = s_w[w];
            wbase += (w < wid) ? n : 0;
            tot += n;
        }
        const int pos = off + wbase + __popc(m & ((1u << lane) - 1u));
        if (f) {
            if (pos >= 0 && pos < n2) I.acell[pos] = c;
            else bad = 1;
        }
        off += tot;
        __syncthreads();
    }
    if (!(total >= 0.0 && total <= (double)n2)) bad = 1;
    if (bad) atomicExch(T.abort_all, 1);      // an inconsistent team count: fail the launch
    if (T.cta == 0 && threadIdx.x == 0) {
        I.acell[n2] = bad ? 0 : (int)total;
        I.out->n_active = I.acell[n2];
    }
    return team_barrier(T) && !bad;
}

__device__ __noinline__ bool phase_classify(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool energy = (P.ssa_solver == YGPU_SSA_ENERGY);
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    const unsigned bb = G.bb;
    // pass 1: kind and partner
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        const int pl = (u >= n2) ? 1 : 0, c = u - pl * n2, i = c % nx, j = c / nx;
        const int mask = pl ? I.mask_y[c] : I.mask_x[c];
        const double uval = pl ? I.u_y[c] : I.u_x[c];
        int kind, part = -1;
        double dv = 0.0;
        if (energy) {
            kind = DOF_FREE;
            auto edge = [&](bool fr, int inner) {
                if (fr) { kind = DOF_TIED; part = inner; } else { kind = DOF_DIR; part = -1; }
            };
            if (mask == 0) kind = DOF_DIR;
            else if (mask == -1) { kind = DOF_DIR; dv = uval; }
            else if (pl == 0) {
                if (i == 0 && !bper(bb, 2)) edge(bfree(bb, 2), 1 + nx * j);
                else if (i == nx - 1 && !bper(bb, 0)) edge(bfree(bb, 0), nx - 2 + nx * j);
                else if (j == 0 && !bper(bb, 3)) edge(bfree(bb, 3), i + nx * 1);
                else if (j == ny - 1 && !bper(bb, 1)) edge(bfree(bb, 1), i + nx * (ny - 2));
            } else {
                if (j == 0 && !bper(bb, 3)) edge(bfree(bb, 3), n2 + i + nx * 1);
                else if (j == ny - 1 && !bper(bb, 1)) edge(bfree(bb, 1), n2 + i + nx * (ny - 2));
                else if (i == 0 && !bper(bb, 2)) edge(bfree(bb, 2), n2 + 1 + nx * j);
                else if (i == nx - 1 && !bper(bb, 0)) edge(bfree(bb, 0), n2 + nx - 2 + nx * j);
            }
            I.ukind[u] = kind;
            I.rpart[u] = part;
            I.dval[u] = dv;
        } else {
            int rk = RROW_INNER;
            if (mask == 0) rk = RROW_ID;
            else if (mask == -1) rk = RROW_ID;
            else {
                // border order: ux left, right, lower, upper; uy lower, upper, left, right
                int side[4], partner[4];
                if (pl == 0) {
                    side[0] = 2; partner[0] = 1 + nx * j;
                    side[1] = 0; partner[1] = nx - 2 + nx * j;
                    side[2] = 3; partner[2] = i + nx * 1;
                    side[3] = 1; partner[3] = i + nx * (ny - 2);
                } else {
                    side[0] = 3; partner[0] = n2 + i + nx * 1;
                    side[1] = 1; partner[1] = n2 + i + nx * (ny - 2);
                    side[2] = 2; partner[2] = n2 + 1 + nx * j;
                    side[3] = 0; partner[3] = n2 + nx - 2 + nx * j;
                }
                bool at[4];
                if (pl == 0) { at[0] = (i == 0); at[1] = (i == nx - 1); at[2] = (j == 0); at[3] = (j == ny - 1); }
                else { at[0] = (j == 0); at[1] = (j == ny - 1); at[2] = (i == 0); at[3] = (i == nx - 1); }
                bool done = false;
                for (int s = 0; s < 4 && !done; s++) {
                    if (at[s] && !bper(bb, side[s])) {
                        done = true;
                        if (bfree(bb, side[s])) { rk = RROW_FREESLIP; part = partner[s]; }
                        else rk = RROW_ID;
                    }
                }
                if (!done && mask == 3) rk = RROW_FRONT;
            }
            I.ukind[u] = rk;
            I.rpart[u] = part;
            I.emap[u] = u;
        }
    }
    if (!energy) return team_barrier(T) && build_active_cells(I, G, T, false);
    if (!team_barrier(T)) return false;
    // pass 2: resolve tied chains to their free root (depth <= 8)
    double bad = 0.0;
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        int m = u, depth = 0;
        while (I.ukind[m] == DOF_TIED) {
            m = I.rpart[m];
            if (++depth > 8) { bad = 1.0; break; }
        }
        I.emap[u] = m;     // root for now
    }
    if (!team_allreduce(T, &bad, 1)) return false;
    if (bad > 0.0) return false;
    // pass 3: a tied unknown whose root is Dirichlet is Dirichlet (value of the root)
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        int k = I.ukind[u];
        if (k == DOF_TIED) {
            int r = I.emap[u];
            if (I.ukind[r] == DOF_DIR) {
                I.dval[u] = I.dval[r];
                I.rpart[u] = -2;     // mark: becomes Dirichlet
            }
        }
    }
    if (!team_barrier(T)) return false;
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        if (I.rpart[u] == -2) {
            I.ukind[u] = DOF_DIR;
            I.rpart[u] = -1;
        }
    }
    if (!team_barrier(T)) return false;
    // pass 4: column map (free: self, tied: root, Dirichlet: -1) and member lists
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        int k = I.ukind[u];
        int r = I.emap[u];
        if (k == DOF_DIR) I.emap[u] = -1;
        else if (k == DOF_FREE) I.emap[u] = u;
        else I.emap[u] = r;
        (void)r;
    }
    if (!team_barrier(T)) return false;
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        int* mem = I.mem + 3 * u;
        mem[0] = mem[1] = mem[2] = -1;
        if (I.ukind[u] != DOF_FREE) continue;
        const int pl = (u >= n2) ? 1 : 0, c = u - pl * n2, i = c % nx, j = c / nx;
        int nm = 0;
        // tied unknowns of the same plane within one cell of the root, in unknown order
        for (int dj = -1; dj <= 1; dj++)
            for (int di = -1; di <= 1; di++) {
                int a = i + di, b = j + dj;
                if (a < 0 || a >= nx || b < 0 || b >= ny || (di == 0 && dj == 0)) continue;
                int t = pl * n2 + a + nx * b;
                if (I.ukind[t] == DOF_TIED && I.emap[t] == u && nm < 3) mem[nm++] = t;
            }
    }
    if (!team_barrier(T)) return false;
    // pass 5: interior fast-path flag (rpart = 1): a free row without members
    // whose four elements exist and hold only free, self-mapped unknowns
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        int fast = 0;
        if (I.ukind[u] == DOF_FREE && I.mem[3 * u] < 0) {
            const int pl = (u >= n2) ? 1 : 0, c = u - pl * n2, i = c % nx, j = c / nx;
            fast = 1;
            for (int e = 0; e < 4 && fast; e++) {
                int ci, cj, d[4];
                if (e < 2) {            // cells
                    ci = (pl == 0) ? i + e : i;
                    cj = (pl == 0) ? j : j + e;
                    if (!elem_index(ci, nx, G.per_x) || !elem_index(cj, ny, G.per_y)) { fast = 0; break; }
                    d[0] = dof_u(G, ci - 1, cj, 0); d[1] = dof_u(G, ci, cj, 0);
                    d[2] = dof_u(G, ci, cj - 1, 1); d[3] = dof_u(G, ci, cj, 1);
                } else {                // corners
                    ci = (pl == 0) ? i : i - (e - 2);
                    cj = (pl == 0) ? j - (e - 2) : j;
                    if (!elem_index(ci, nx, G.per_x) || !elem_index(cj, ny, G.per_y)) { fast = 0; break; }
                    d[0] = dof_u(G, ci, cj, 0); d[1] = dof_u(G, ci, cj + 1, 0);
                    d[2] = dof_u(G, ci, cj, 1); d[3] = dof_u(G, ci + 1, cj, 1);
                }
                // a column may be a free unknown or a Dirichlet unknown of value 0:
                // Krylov vectors and the iterate are exactly 0 on those rows
                for (int q = 0; q < 4; q++) {
                    const int dq = d[q];
                    if (dq < 0) { fast = 0; break; }
                    const bool self = (I.emap[dq] == dq);
                    const bool zero_dir = (I.ukind[dq] == DOF_DIR && I.dval[dq] == 0.0);
                    if (!self && !zero_dir) { fast = 0; break; }
                }
            }
        }
        I.rpart[u] = fast;
    }
    return team_barrier(T) && build_active_cells(I, G, T, true);
}

// ---------------------------------------------------------------------------
// Phase: linear system -- rhs, start vector, Jacobi diagonal (FP64)
// ---------------------------------------------------------------------------
// -p ilu on the residual form: BiCGSTAB with the ILU(0) factors, in FP64 in both
// precisions. Warm-started from the last Picard iterate it needs a few
// iterations per linear solve, where the mixed mode's FP32 inner solves would
// only add defect-correction steps (the FP32 coefficients stay as they are).
YG_DEV bool krylov_fp64_ilu(const Inst& I, const ygpu_dyn_par& P, const Geo& G) {
    return P.ssa_solver != YGPU_SSA_ENERGY && P.lin_precond == YGPU_PRE_ILU0 && I.icol && I.ilu && ilu_colourable(G);
}
__device__ __noinline__ void phase_system(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T, double& bnorm2) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool energy = (P.ssa_solver == YGPU_SSA_ENERGY);
    const bool drag = (P.ssa_vel_lim_method == YGPU_VEL_LIM_DRAG);
    const int n2 = G.n2, nx = G.nx, ny = G.ny;
    const double* N = I.visc_int;
    const OpK<double> K64 = make_opk<double>(G);
    const bool ilu64 = krylov_fp64_ilu(I, P, G);     // the FP64 BiCGSTAB of -p ilu reads the FP64 diagonal too
    double bn2 = 0.0;
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        const int pl = (u >= n2) ? 1 : 0, c = u - pl * n2;
        const double uval = pl ? I.u_y[c] : I.u_x[c];
        double b, x0, d = 1.0;
        if (energy) {
            const int k = I.ukind[u];
            if (k == DOF_DIR) { b = I.dval[u]; x0 = I.dval[u]; }
            else if (k == DOF_TIED) { b = 0.0; x0 = 0.0; }
            else {
                // forcing of the root and its members, minus the lifted Dirichlet columns
                b = 0.0;
                d = 0.0;
                const int* mem = I.mem + 3 * u;
                // interior rows (no members, only free or zero-Dirichlet columns):
                // nothing to lift, and the diagonal of the 9-point stencil in closed form
                const bool fast = (I.rpart[u] == 1);
                if (fast) {
                    const int i = c % nx, j = c / nx;
                    const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
                    const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
                    const double Ni = N[c], Bc = I.Nab[c];
                    if (pl == 0) {
                        const double Np = N[ip1 + nx * j], Bm = I.Nab[i + nx * jm1];
                        d = 4.0 * K64.dyodx * (Np + Ni) + K64.dxody * (Bc + Bm) + I.drag_x[c];
                    } else {
                        const double Np = N[i + nx * jp1], Bm = I.Nab[im1 + nx * j];
                        d = 4.0 * K64.dxody * (Np + Ni) + K64.dyodx * (Bc + Bm) + I.drag_y[c];
                    }
                }
                for (int m = -1; m < 3; m++) {
                    int mm = (m < 0) ? u : mem[m];
                    if (mm < 0) break;
                    const int mpl = (mm >= n2) ? 1 : 0, mc = mm - mpl * n2, mi = mc % nx, mj = mc / nx;
                    const int mask = mpl ? I.mask_y[mc] : I.mask_x[mc];
                    const double w = (mask == 3 || mask == 4) ? 0.5 : 1.0;
                    if (drag) b = b + w * (mpl ? I.lr_y[mc] : I.lr_x[mc]) * G.dxdy;
                    if (mask == 3) {
                        int ipj = mpl ? mi + nx * ((mj == ny - 1) ? 0 : mj + 1) : ((mi == nx - 1) ? 0 : mi + 1) + nx * mj;
                        double tl = mpl ? I.taul_y[mc] : I.taul_x[mc];
                        double dl = mpl ? G.dx : G.dy;
                        if (I.f_ice[mc] == 1.0 && I.f_ice[ipj] < 1.0) b = b + tl * dl;
                        else b = b - tl * dl;
                    } else {
                        b = b - (mpl ? I.taud_y[mc] : I.taud_x[mc]) * G.dxdy;
                    }
                    if (fast) break;         // forcing done; diagonal above
                    auto lift = [&](int dd) -> double {
                        if (dd < 0) return 0.0;
                        return (I.ukind[dd] == DOF_DIR) ? I.dval[dd] : 0.0;
                    };
                    b = b - member_elems<double>(G, K64, N, I.Nab, mm, lift);
                    auto unit = [&](int dd) -> double {
                        if (dd < 0) return 0.0;
                        return (I.emap[dd] == u) ? 1.0 : 0.0;
                    };
                    d = d + (mpl ? I.drag_y[mc] : I.drag_x[mc]) + member_elems<double>(G, K64, N, I.Nab, mm, unit);
                }
                x0 = uval;
            }
        } else {
            const int rk = I.ukind[u];
            const int mask = pl ? I.mask_y[c] : I.mask_x[c];
            if (rk == RROW_ID) {
                b = (mask == -1) ? uval : 0.0;
                x0 = (mask == -1) ? uval : 0.0;
            } else if (rk == RROW_FREESLIP) {
                b = 0.0;
                x0 = uval;
            } else if (rk == RROW_FRONT) {
                b = pl ? I.taul_y[c] : I.taul_x[c];
                x0 = uval;
                residual_row<double, double>(I, G, K64, N, I.Nab, I.drag_x, I.drag_y, I.x, u, &d);
            } else {
                const double w = (mask == 4) ? 0.5 : 1.0;
                double lr = drag ? w * (pl ? I.lr_y[c] : I.lr_x[c]) : 0.0;
                b = (pl ? I.taud_y[c] : I.taud_x[c]) - lr;
                x0 = uval;
                residual_row<double, double>(I, G, K64, N, I.Nab, I.drag_x, I.drag_y, I.x, u, &d);
            }
        }
        // identity rows start at their solution (x = b) also with -initx_zeros:
        // the Krylov loops skip cells whose two rows are identity
        const bool ident = energy ? (I.ukind[u] != DOF_FREE) : (I.ukind[u] == RROW_ID);
        if (P.lin_initx_zeros && !ident) x0 = 0.0;
        if (ident) x0 = b;
        I.b[u] = b;
        I.x[u] = x0;
        // the Jacobi diagonal: FP64 for the FP64 solvers; the mixed mode's FP32
        // inner solves take an FP32 reciprocal (no FP64 division)
        if (I.fdinv) {
            const float df = (float)d;
            I.fdinv[u] = (df != 0.0f) ? 1.0f / df : 1.0f;
        }
        if (!I.fdinv || ilu64) I.dinv[u] = (d != 0.0) ? 1.0 / d : 1.0;
        bn2 += b * b;
    }
    bnorm2 = bn2;
}

// ---------------------------------------------------------------------------
// Krylov solvers (team-parallel, deterministic reductions)
// ---------------------------------------------------------------------------
// CG with Jacobi (x updated in place). Returns LIS status; iters/relres out.
template <typename T, typename Op, typename CT>
__device__ __noinline__ int krylov_cg(Team& Tm_, int nu, const Op& A, const CT* dinv, T* x, const T* b, T* r, T* p, T* q, T* z,
                     int maxiter, double tol, double bnrm, bool precond, int& iters, double& relres, bool& ok) {
    TeamLocal tl_(Tm_);
    Team& Tm = tl_.t;
    ok = true;
    iters = 0;
    // r = b - A x
    A(Tm, x, q);
    double red[2] = {0.0, 0.0};
    for (int u = Tm.tid; u < nu; u += Tm.nthr) {
        T ru = b[u] - q[u];
        r[u] = ru;
        T zu = precond ? (T)dinv[u] * ru : ru;
        z[u] = zu;
        p[u] = zu;
        red[0] += (double)ru * (double)ru;
        red[1] += (double)ru * (double)zu;
    }
    if (!(ok = team_allreduce(Tm, red, 2))) return YGPU_ERR_TIMEOUT;
    relres = sqrt(red[0]) / bnrm;
    if (relres <= tol) return YGPU_OK;
    double rz = red[1];
    for (int it = 1; it <= maxiter; it++) {
        A(Tm, p, q);
        double pq = 0.0;
        for (int u = Tm.tid; u < nu; u += Tm.nthr) pq += (double)p[u] * (double)q[u];
        if (!(ok = team_allreduce(Tm, &pq, 1))) return YGPU_ERR_TIMEOUT;
        iters = it;
        if (pq == 0.0 || !isfinite(pq)) return YGPU_BREAKDOWN;
        const double alpha = rz / pq;
        double rr[2] = {0.0, 0.0};
        for (int u = Tm.tid; u < nu; u += Tm.nthr) {
            x[u] = x[u] + (T)alpha * p[u];
            T ru = r[u] - (T)alpha * q[u];
            r[u] = ru;
            T zu = precond ? (T)dinv[u] * ru : ru;
            z[u] = zu;
            rr[0] += (double)ru * (double)ru;
            rr[1] += (double)ru * (double)zu;
        }
        if (!(ok = team_allreduce(Tm, rr, 2))) return YGPU_ERR_TIMEOUT;
        relres = sqrt(rr[0]) / bnrm;
        if (relres <= tol) return YGPU_OK;
        const double beta = rr[1] / rz;
        rz = rr[1];
        for (int u = Tm.tid; u < nu; u += Tm.nthr) p[u] = z[u] + (T)beta * p[u];
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
    }
    return YGPU_MAXITER;
}

// Pipelined preconditioned CG (Ghysels and Vanroose 2014): one team
// all-reduce per iteration. The three dot products of an iteration are reduced
// together, and the operator apply, preconditioner and eight vector updates of
// a row are fused into one pass. The operator input m ping-pongs between two
// buffers because rows read it at their neighbours while it is being renewed.
// The recursively updated residual is checked against b - A x when it reaches
// the tolerance; if the true residual is above it, the recursion restarts from
// the true residual.

// 1/b for the recurrence scalars of the Krylov methods. FP32: the division.
// FP64: the FP32 reciprocal refined by two Newton steps, y <- y + y (1 - b y),
// each squaring the relative error (about 1e-7 from the seed), to within a few
// ulp in about six dependent operations where the IEEE division takes a longer
// chain on this part's FP64 pipe; the division where b is outside FP32's
// normal range.
YG_DEV float scalar_rcp(float b) { return 1.0f / b; }
YG_DEV double scalar_rcp(double b) {
    const float bf = fabsf((float)b);
    if (!(bf >= 1.17549435e-38f && bf <= 3.4e38f)) return 1.0 / b;
    double y = (double)__frcp_rn((float)b);
    double e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    return fma(y, e, y);
}

template <typename T, typename Op, typename CT>
__device__ __noinline__ int krylov_pcg_pipe(Team& Tm_, int nu, const Op& A, const CT* __restrict__ dinv,
                                            T* __restrict__ x, const T* __restrict__ b, T* __restrict__ r,
                                            T* __restrict__ u, T* __restrict__ w, T* m0, T* m1, T* __restrict__ z,
                                            T* __restrict__ q, T* __restrict__ s, T* __restrict__ p, int maxiter,
                                            double tol, double bnrm, bool precond, int& iters, double& relres,
                                            bool& ok) {
    TeamLocal tl_(Tm_);
    Team& Tm = tl_.t;
    // Scalar recurrences run on one thread per CTA and are broadcast through
    // shared memory: FP64 division and square root are slow on this part, and
    // every thread of the team would otherwise repeat them.
    // The all-reduced sums and the scalars are in T: an FP32 inner solve keeps
    // its whole iteration off the FP64 pipe (relres leaves as FP64 on exit only).
    __shared__ T s_ab[3];          // alpha, beta, relres
    __shared__ int s_flag;         // 0 continue, 1 converged, 2 breakdown
    const bool lead = (threadIdx.x == 0);
    using W = T;                   // precision of the scalar recurrences
    ok = true;
    iters = 0;
    auto Mi = [&](int k) -> T { return precond ? (T)dinv[k] : T(1); };
    // Work items of the iteration loop: cells (FP32, both rows of a cell per
    // item) or rows (FP64), over the active cells when the operator has a list.
    // The first YG_ITEM_CACHE items of each thread are looked up once per
    // call and kept in shared memory (thread-private slots).
    const bool by_cell = (sizeof(T) == sizeof(float));
    const int n2 = A.n2();
    const int nact = A.acell ? min(max(A.acell[n2], 0), n2) : n2;
    const int nitem = by_cell ? nact : 2 * nact;
    auto item = [&](int t) -> int {
        if (!A.acell) return t;
        if (by_cell || t < nact) return A.acell[t];
        return n2 + A.acell[t - nact];
    };
    int* s_item = g_item_cache;
    const int cache = (blockDim.x <= YG_ITEM_BLOCK) ? YG_ITEM_CACHE : 0;
    // each CTA takes one contiguous chunk of the work items
    const int chunk = (nitem + Tm.ncta - 1) / Tm.ncta;
    const int t_beg = min(Tm.cta * chunk, nitem), t_end = min(t_beg + chunk, nitem);
    const int t0 = t_beg + (int)threadIdx.x, tstep = (int)blockDim.x;
    {
        int q = 0;
        for (int t = t0; t < t_end && q < cache; t += tstep, q++) s_item[q * blockDim.x + threadIdx.x] = item(t);
    }
    int it = 0;
    for (int restart = 0; restart < 8; restart++) {
        // r = b - A x, u = M r
        for (int k = Tm.tid; k < nu; k += Tm.nthr) {
            T rk = b[k] - A.row(k, x);
            r[k] = rk;
            u[k] = Mi(k) * rk;
        }
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
        // w = A u; partial dots; m = M w. Per-thread partial sums in the working
        // precision (FP32 accumulation in the inner solve of the mixed mode),
        // combined across the team in FP64.
        T a0 = T(0), a1 = T(0), a2 = T(0);
        for (int k = Tm.tid; k < nu; k += Tm.nthr) {
            T wk = A.row(k, u);
            w[k] = wk;
            const T mk = Mi(k) * wk;
            m0[k] = mk;
            m1[k] = T(0);
            z[k] = T(0); q[k] = T(0); s[k] = T(0); p[k] = T(0);
            const T rk = r[k], uk = u[k];
            a0 += rk * uk;
            a1 += wk * uk;
            a2 += rk * rk;
        }
        T red[3];
        {
            const T part[3] = {a0, a1, a2};
            if (!(ok = team_allreduce_w<T>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
        }
        // lead thread: the reciprocals of gam and alpha carried by the recurrence
        // (alpha = gam / t with t = del - beta gam / alpha_old, so 1 / alpha =
        // t / gam); s_ab[2] holds ||r||^2, compared with (tol ||b||)^2
        W inv_gam_old = W(1), inv_alpha_old = W(1);
        const W tol2 = ((W)tol * (W)bnrm) * ((W)tol * (W)bnrm);
        auto rel_of = [&](W rr) -> double { return (double)(sqrt(rr) / (W)bnrm); };
        if (lead) {
            const W rr = red[2];
            s_ab[2] = rr;
            // a non-finite norm (an Inf or NaN right-hand side) breaks down below
            if (isfinite(rr) && rr <= tol2) s_flag = 1;
            else {
                const W gam = red[0], del = red[1];
                const W inv_gam = scalar_rcp(gam);
                const W alpha = gam * scalar_rcp(del);
                if (!isfinite(alpha) || del == W(0)) s_flag = 2;
                else {
                    s_flag = 0;
                    s_ab[0] = alpha;
                    s_ab[1] = W(0);
                    inv_gam_old = inv_gam;
                    inv_alpha_old = del * inv_gam;
                }
            }
        }
        __syncthreads();
        if (s_flag == 1) { relres = rel_of(s_ab[2]); iters = it; return YGPU_OK; }
        if (s_flag == 2) { relres = rel_of(s_ab[2]); iters = it; return (it < maxiter) ? YGPU_BREAKDOWN : YGPU_MAXITER; }
        T* mc = m0;
        T* mn = m1;
        bool recheck = false;
        while (it < maxiter) {
            const T a = s_ab[0], bt = s_ab[1];
            a0 = a1 = a2 = T(0);
            // one row's loads (operator row, nine vectors, preconditioner)
            struct RowIn { T n, m, z, q, s, p, x, r, u, w, mi; };
            auto load = [&](int k, T nk) {
                RowIn R;
                R.n = nk;
                R.m = mc[k]; R.z = z[k]; R.q = q[k]; R.s = s[k]; R.p = p[k];
                R.x = x[k]; R.r = r[k]; R.u = u[k]; R.w = w[k]; R.mi = Mi(k);
                return R;
            };
            auto update = [&](int k, const RowIn& R) {
                const T zk = R.n + bt * R.z;
                const T qk = R.m + bt * R.q;
                const T sk = R.w + bt * R.s;
                const T pk = R.u + bt * R.p;
                z[k] = zk; q[k] = qk; s[k] = sk; p[k] = pk;
                x[k] = R.x + a * pk;
                const T rk = R.r - a * sk;
                const T uk = R.u - a * qk;
                const T wk = R.w - a * zk;
                r[k] = rk; u[k] = uk; w[k] = wk;
                mn[k] = R.mi * wk;
                a0 += rk * uk;
                a1 += wk * uk;
                a2 += rk * rk;
            };
            // one cell per thread and trip: both of its rows' loads (the shared
            // stencil loads included) precede either row's stores. Rows c and
            // n2 + c belong to the thread of cell c here; every use of these
            // vectors with the row-k-per-thread-k mapping (restart, true
            // residual, the caller) follows a team all-reduce.
            // With an active-cell list the cells whose two rows are identity are
            // skipped: all their vectors are zero (m1 included) and x = b there.
            int q = 0;
            for (int t = t0; t < t_end; t += tstep, q++) {
                const int k = (q < cache) ? s_item[q * blockDim.x + threadIdx.x] : item(t);
                if (by_cell) {
                    const int j = k / A.nx(), i = k - j * A.nx();
                    T y0, y1;
                    A.cell(k, i, j, mc, y0, y1);
                    const RowIn R0 = load(k, y0);
                    const RowIn R1 = load(n2 + k, y1);
                    update(k, R0);
                    update(n2 + k, R1);
                } else {
                    // FP64: one row per item (the two-row body exceeds the register budget)
                    update(k, load(k, A.row(k, mc)));
                }
            }
            it++;
            {
                const T part[3] = {a0, a1, a2};
                if (!(ok = team_allreduce_w<T>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
            }
            { T* t = mc; mc = mn; mn = t; }
            if (lead) {
                // FP32 inner solves: the recurrence scalars in FP32 (its division
                // and square root are far faster than FP64's on this part); FP64:
                // two independent reciprocals, no division or square root
                const W rr = red[2];
                s_ab[2] = rr;
                if (!isfinite(rr)) s_flag = 2;
                else if (rr <= tol2) s_flag = 1;
                else {
                    const W gam = red[0], del = red[1];
                    const W inv_gam = scalar_rcp(gam);
                    const W beta = gam * inv_gam_old;
                    const W t = del - beta * gam * inv_alpha_old;
                    const W alpha = gam * scalar_rcp(t);
                    if (!isfinite(alpha) || !isfinite(beta) || del == W(0)) s_flag = 3;
                    else {
                        s_flag = 0;
                        s_ab[0] = alpha;
                        s_ab[1] = beta;
                        inv_gam_old = inv_gam;
                        inv_alpha_old = t * inv_gam;
                    }
                }
            }
            __syncthreads();
            // s_flag / s_ab are rewritten only after the next all-reduce's first
            // __syncthreads, so every thread has read them by then
            const int flag = s_flag;
            if (flag != 0) relres = rel_of(s_ab[2]);
            if (flag == 2) { iters = it; return YGPU_BREAKDOWN; }
            if (flag == 1) { recheck = true; break; }
            if (flag == 3) {
                // the next iteration's coefficients broke down
                if (it < maxiter) { iters = it; return YGPU_BREAKDOWN; }
                break;
            }
        }
        iters = it;
        relres = rel_of(s_ab[2]);
        if (!recheck) return YGPU_MAXITER;
        // true residual check (in T, as the recurrence)
        T tr = T(0);
        for (int k = Tm.tid; k < nu; k += Tm.nthr) {
            const T rk = b[k] - A.row(k, x);
            tr += rk * rk;
        }
        {
            T trs;
            if (!(ok = team_allreduce_w<T>(Tm, &tr, &trs, 1))) return YGPU_ERR_TIMEOUT;
            tr = trs;
        }
        relres = (double)(sqrt(tr) / (W)bnrm);
        if (relres <= tol) return YGPU_OK;
        if (it >= maxiter) return YGPU_MAXITER;
    }
    return YGPU_MAXITER;
}

// Pipelined preconditioned CG of the FP32 inner solves (energy form), the
// same recurrence as krylov_pcg_pipe laid out for this part's memory system:
//  - the eight recurrence vectors of an unknown are one 32-byte record of two
//    float4, (z, q, s, p) and (x, r, u, w): a row's state moves in two vector
//    loads and two vector stores;
//  - each thread's active cells are cached in shared memory packed with their
//    grid position and row kinds (i | j << 14 | kind(ux) << 28 | kind(uy) << 30),
//    so an iteration reads no cell list or row kind and divides nothing;
//  - a cell's state loads are issued before its stencil loads, which do not
//    depend on them: one memory round trip per cell;
//  - identity rows (Dirichlet or tied) are skipped: all their vectors stay 0.
// It is the inner solve of the mixed defect correction: A d = r64 * rs from
// d = 0, and x64 += d * xs when the recurrence stops, with no true-residual
// check or restart (the caller's next FP64 residual checks every correction).
// r64 must be zero outside the non-identity rows of the active cells. Only the
// operator input m and the first pass's u (both read at neighbouring cells) live
// in plain arrays. Needs nx, ny < 2^14.
// Shared-memory row records of the FP32 cell CG: a thread's first S cells keep
// their four float4 records (two per row) in dynamic shared memory for the whole
// recurrence; slot (q, f) of a thread at (q * 4 + f) * blockDim.x + threadIdx.x
// (consecutive threads on consecutive 16-byte words). S follows from the dynamic
// shared memory of the launch (none: every record in global memory).
#define YG_KREC_MAX 4
extern __shared__ float4 g_krec[];
YG_DEV int krec_slots() {
    unsigned dsm;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dsm));
    const int n = (int)(dsm / (4u * sizeof(float4) * blockDim.x));
    return n < YG_KREC_MAX ? n : YG_KREC_MAX;
}
YG_DEV float4& krec(int q, int f) { return g_krec[(q * 4 + f) * blockDim.x + threadIdx.x]; }

YG_DEV unsigned cell_pack(int i, int j, unsigned k0, unsigned k1) {
    return (unsigned)i | ((unsigned)j << 14) | (k0 << 28) | (k1 << 30);
}
template <typename Op>
__device__ __noinline__ int krylov_pcg_cells(Team& Tm_, int nu, const Op& A, const float* __restrict__ dinv,
                                             double* __restrict__ x64, double xs, const double* __restrict__ r64,
                                             double rs, float* __restrict__ u, float* m0, float* m1,
                                             float4* __restrict__ st, int maxiter, double tol, bool precond,
                                             int& iters, double& relres, bool& ok) {
    // no register copy of the team here: the cell loop needs the registers
    Team& Tm = Tm_;
    __shared__ float s_ab[3];      // alpha, beta, relres
    __shared__ int s_flag;         // 0 continue, 1 converged, 2 breakdown, 3 next coefficients broke down
    const bool lead = (threadIdx.x == 0);
    ok = true;
    iters = 0;
    auto Mi = [&](int k) -> float { return precond ? dinv[k] : 1.0f; };
    // everything the iterations read besides the vectors is copied to registers
    // here: the team, the grid and the operator live in local memory, and reads
    // of them inside the loop would be repeated after every store (the stores
    // could alias them) and would miss the L1, which each team barrier's
    // acquire invalidates
    const int tid = Tm.tid, nthr = Tm.nthr;
    const Geo Gv = *A.G;
    const OpK<float> Kv = A.K;
    const float* __restrict__ cN = A.N;
    const float* __restrict__ cNab = A.Nab;
    const float* __restrict__ cdgx = A.dgx;
    const float* __restrict__ cdgy = A.dgy;
    const int n2 = Gv.n2, nx = Gv.nx;
    const int nact = A.acell ? min(max(A.acell[n2], 0), n2) : n2;
    auto pack = [&](int t) -> unsigned {
        const int c = A.acell ? A.acell[t] : t;
        const int j = c / nx, i = c - j * nx;
        return cell_pack(i, j, A.row_kind(c), A.row_kind(n2 + c));
    };
    int* s_item = g_item_cache;
    const int cache = (blockDim.x <= YG_ITEM_BLOCK) ? YG_ITEM_CACHE : 0;
    // each CTA takes one contiguous chunk of the active-cell list (every SM of the
    // team gets cells, and neighbouring threads take neighbouring cells)
    const int chunk = (nact + Tm.ncta - 1) / Tm.ncta;
    const int t_beg = min(Tm.cta * chunk, nact), t_end = min(t_beg + chunk, nact);
    const int t0 = t_beg + (int)threadIdx.x, tstep = (int)blockDim.x;
    const int S = min(krec_slots(), cache);     // cells whose records stay in shared memory
    {
        int q = 0;
        for (int t = t0; t < t_end && q < cache; t += tstep, q++) s_item[q * blockDim.x + threadIdx.x] = (int)pack(t);
    }
    // x64 += d * xs on the non-identity rows of the thread's cells (FP64
    // accumulation), then a team barrier (the caller reads x64 at every row)
    auto flush_x = [&]() -> bool {
        int q = 0;
        for (int t = t0; t < t_end; t += tstep, q++) {
            const unsigned pk = (q < cache) ? (unsigned)s_item[q * blockDim.x + threadIdx.x] : pack(t);
            const int c = (int)(pk & 0x3fffu) + nx * (int)((pk >> 14) & 0x3fffu);
            if (((pk >> 28) & 3u) != 1u) {
                const float d = (q < S) ? krec(q, 1).x : st[2 * c + 1].x;
                x64[c] = x64[c] + (double)d * xs;
            }
            if ((pk >> 30) != 1u) {
                const float d = (q < S) ? krec(q, 3).x : st[2 * (n2 + c) + 1].x;
                x64[n2 + c] = x64[n2 + c] + (double)d * xs;
            }
        }
        return team_barrier(Tm);
    };
    int it = 0;
    {
        // u = M r with r = r64 * rs (d = 0: r is the right-hand side), m = 0, on
        // every row (identity rows keep u = m = 0)
        for (int k = tid; k < nu; k += nthr) {
            u[k] = Mi(k) * (float)(r64[k] * rs);
            m0[k] = 0.0f;
            m1[k] = 0.0f;
        }
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
        // w = A u on the non-identity rows of the thread's cells, m = M w, the
        // row records (the first S cells' in shared memory), partial dots
        float a0 = 0.0f, a1 = 0.0f, a2 = 0.0f;
        auto init = [&](int k, float wk, float4* R0, float4* R1) {
            const float rk = (float)(r64[k] * rs), uk = u[k];
            m0[k] = Mi(k) * wk;
            *R0 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
            *R1 = make_float4(0.0f, rk, uk, wk);
            a0 += rk * uk;
            a1 += wk * uk;
            a2 += rk * rk;
        };
        {
            int q = 0;
            for (int t = t0; t < t_end; t += tstep, q++) {
                const unsigned pk = (q < cache) ? (unsigned)s_item[q * blockDim.x + threadIdx.x] : pack(t);
                const int i = (int)(pk & 0x3fffu), j = (int)((pk >> 14) & 0x3fffu);
                const unsigned k0 = (pk >> 28) & 3u, k1 = pk >> 30;
                const int c = i + nx * j, c1 = n2 + c;
                const bool sh = q < S;
                if (k0 == 0u || k1 == 0u) {
                    float y0, y1;
                    energy_cell_fast<float, float>(Gv, Kv, cN, cNab, cdgx, cdgy, u, c, i, j, y0, y1);
                    if (k0 == 0u) init(c, y0, sh ? &krec(q, 0) : &st[2 * c], sh ? &krec(q, 1) : &st[2 * c + 1]);
                    if (k1 == 0u) init(c1, y1, sh ? &krec(q, 2) : &st[2 * c1], sh ? &krec(q, 3) : &st[2 * c1 + 1]);
                }
#pragma unroll 1
                for (int h = 0; h < 2; h++) {
                    if (((h == 0) ? k0 : k1) != 2u) continue;
                    const int k = c + h * n2;
                    init(k, A.general(k, u), sh ? &krec(q, 2 * h) : &st[2 * k], sh ? &krec(q, 2 * h + 1) : &st[2 * k + 1]);
                }
            }
        }
        float red[3];
        {
            const float part[3] = {a0, a1, a2};
            if (!(ok = team_allreduce_w<float>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
        }
        float gam_old = 1.0f, alpha_old = 1.0f;
        if (lead) {
            const float rel = sqrtf(red[2]);     // the right-hand side has unit norm
            s_ab[2] = rel;
            if (rel <= (float)tol) s_flag = 1;
            else {
                const float gam = red[0], del = red[1];
                const float alpha = gam / del;
                if (!isfinite(alpha) || del == 0.0f) s_flag = 2;
                else {
                    s_flag = 0;
                    s_ab[0] = alpha;
                    s_ab[1] = 0.0f;
                    gam_old = gam;
                    alpha_old = alpha;
                }
            }
        }
        __syncthreads();
        if (s_flag == 1) { relres = (double)s_ab[2]; iters = it; return YGPU_OK; }
        if (s_flag == 2) { relres = (double)s_ab[2]; iters = it; return (it < maxiter) ? YGPU_BREAKDOWN : YGPU_MAXITER; }
        float* mc = m0;
        float* mn = m1;
        bool converged = false;
        int exit_st = YGPU_MAXITER;
        while (it < maxiter) {
            const float a = s_ab[0], bt = s_ab[1];
            a0 = a1 = a2 = 0.0f;
            // one row's update from its records, operator value nk and m, M
            auto update = [&](int k, float4& A0, float4& A1, float nk, float mk, float mi, float4* R0, float4* R1) {
                // A0 = (z, q, s, p), A1 = (x, r, u, w)
                const float zk = nk + bt * A0.x;
                const float qk = mk + bt * A0.y;
                const float sk = A1.w + bt * A0.z;
                const float pk = A1.z + bt * A0.w;
                const float xk = A1.x + a * pk;
                const float rk = A1.y - a * sk;
                const float uk = A1.z - a * qk;
                const float wk = A1.w - a * zk;
                *R0 = make_float4(zk, qk, sk, pk);
                *R1 = make_float4(xk, rk, uk, wk);
                mn[k] = mi * wk;
                a0 += rk * uk;
                a1 += wk * uk;
                a2 += rk * rk;
            };
            const float* __restrict__ mcr = mc;
            int q = 0;
            for (int t = t0; t < t_end; t += tstep, q++) {
                const unsigned pk = (q < cache) ? (unsigned)s_item[q * blockDim.x + threadIdx.x] : pack(t);
                const int i = (int)(pk & 0x3fffu), j = (int)((pk >> 14) & 0x3fffu);
                const unsigned k0 = (pk >> 28) & 3u, k1 = pk >> 30;
                const int c = i + nx * j, c1 = n2 + c;
                if (k0 != 0u && k1 != 0u) continue;      // no interior-stencil row
                float4 A0 = make_float4(0.f, 0.f, 0.f, 0.f), A1 = A0, B0 = A0, B1 = A0;
                float m0v = 0.0f, m1v = 0.0f, i0 = 0.0f, i1 = 0.0f;
                const bool sh = q < S;
                float4* ra0 = sh ? &krec(q, 0) : &st[2 * c];
                float4* ra1 = sh ? &krec(q, 1) : &st[2 * c + 1];
                float4* rb0 = sh ? &krec(q, 2) : &st[2 * c1];
                float4* rb1 = sh ? &krec(q, 3) : &st[2 * c1 + 1];
                if (k0 == 0u) { A0 = *ra0; A1 = *ra1; m0v = mcr[c]; i0 = Mi(c); }
                if (k1 == 0u) { B0 = *rb0; B1 = *rb1; m1v = mcr[c1]; i1 = Mi(c1); }
                float y0, y1;
                energy_cell_fast<float, float>(Gv, Kv, cN, cNab, cdgx, cdgy, mcr, c, i, j, y0, y1);
                if (k0 == 0u) update(c, A0, A1, y0, m0v, i0, ra0, ra1);
                if (k1 == 0u) update(c1, B0, B1, y1, m1v, i1, rb0, rb1);
            }
            // rows outside the interior stencil in a second pass: the calls stay
            // out of the main loop (whose live registers they would spill)
            q = 0;
            for (int t = t0; t < t_end; t += tstep, q++) {
                const unsigned pk = (q < cache) ? (unsigned)s_item[q * blockDim.x + threadIdx.x] : pack(t);
                const unsigned k0 = (pk >> 28) & 3u, k1 = pk >> 30;
                if (k0 != 2u && k1 != 2u) continue;
                const int c = (int)(pk & 0x3fffu) + nx * (int)((pk >> 14) & 0x3fffu);
#pragma unroll 1
                for (int h = 0; h < 2; h++) {
                    if (((h == 0) ? k0 : k1) != 2u) continue;
                    const int k = c + h * n2;
                    float4* p0 = (q < S) ? &krec(q, 2 * h) : &st[2 * k];
                    float4* p1 = (q < S) ? &krec(q, 2 * h + 1) : &st[2 * k + 1];
                    float4 R0 = *p0, R1 = *p1;
                    const float mk = mcr[k], mi = Mi(k);
                    update(k, R0, R1, A.general(k, mc), mk, mi, p0, p1);
                }
            }
            it++;
            {
                const float part[3] = {a0, a1, a2};
                if (!(ok = team_allreduce_w<float>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
            }
            { float* tt = mc; mc = mn; mn = tt; }
            if (lead) {
                const float rel = sqrtf(red[2]);
                s_ab[2] = rel;
                if (!isfinite(rel)) s_flag = 2;
                else if (rel <= (float)tol) s_flag = 1;
                else {
                    const float gam = red[0], del = red[1];
                    const float beta = gam / gam_old;
                    const float alpha = gam / (del - beta * gam / alpha_old);
                    if (!isfinite(alpha) || !isfinite(beta) || del == 0.0f) s_flag = 3;
                    else {
                        s_flag = 0;
                        s_ab[0] = alpha;
                        s_ab[1] = beta;
                        gam_old = gam;
                        alpha_old = alpha;
                    }
                }
            }
            __syncthreads();
            // s_flag / s_ab are rewritten only after the next all-reduce's first
            // __syncthreads, so every thread has read them by then
            const int flag = s_flag;
            if (flag == 2) { exit_st = YGPU_BREAKDOWN; break; }
            if (flag == 1) { converged = true; break; }
            if (flag == 3) {
                if (it < maxiter) exit_st = YGPU_BREAKDOWN;
                break;
            }
        }
        relres = (double)s_ab[2];
        iters = it;
        if (!(ok = flush_x())) return YGPU_ERR_TIMEOUT;
        return converged ? YGPU_OK : exit_st;
    }
}

// BiCGSTAB with Jacobi (van der Vorst 1992, as in the oracle). The scalar
// recurrences run on one thread per CTA and are broadcast through shared
// memory (see krylov_pcg_pipe). With an active-cell list the iterations visit
// the rows of the listed cells only: identity rows enter with x = b, so r, rt
// and p are zero there, and p_hat and s_hat (the operator inputs, read at
// neighbouring columns) are cleared on every row at the start.
template <typename T, typename Op, typename CT>
__device__ __noinline__ int krylov_bicgstab(Team& Tm_, int nu, const Op& A, const CT* __restrict__ dinv,
                                            T* __restrict__ x, const T* __restrict__ b, T* __restrict__ r,
                                            T* __restrict__ rt, T* __restrict__ p, T* v, T* __restrict__ s, T* t,
                                            T* ph, T* sh, int maxiter, double tol, double bnrm, bool precond,
                                            int& iters, double& relres, bool& ok, const IluM<T>* M = nullptr) {
    TeamLocal tl_(Tm_);
    Team& Tm = tl_.t;
    // sums and scalars in T (an FP32 inner solve stays off the FP64 pipe)
    __shared__ T s_sc[4];          // alpha, omega, beta, relres
    __shared__ int s_flag;         // 0 continue, 1 converged, 2 breakdown
    const bool lead = (threadIdx.x == 0);
    using W = T;                   // precision of the scalar recurrences (FP32 in the inner solves)
    ok = true;
    iters = 0;
    A(Tm, x, v);
    T a0 = T(0);
    for (int u = Tm.tid; u < nu; u += Tm.nthr) {
        T ru = b[u] - v[u];
        r[u] = ru;
        rt[u] = ru;
        p[u] = T(0);
        ph[u] = T(0);
        sh[u] = T(0);
        s[u] = T(0);       // the ILU(0) solves read s on every row, the loops write active rows only
        a0 += ru * ru;
    }
    T red[1];
    if (!(ok = team_allreduce_w<T>(Tm, &a0, red, 1))) return YGPU_ERR_TIMEOUT;
    // rows of this thread in the iterations (its own cache slots)
    const RowItems R = make_row_items(Tm, op_acell(A), A.n2(), nu);
    // lead-thread state of the recurrence
    W rho = red[0], rho_old = W(1), alpha = W(1), omega = W(1);     // (rt, r) with rt = r
    if (lead) {
        s_sc[3] = sqrt(red[0]) / (W)bnrm;
        s_flag = (s_sc[3] <= (W)tol) ? 1 : 0;
    }
    __syncthreads();
    relres = (double)s_sc[3];
    if (s_flag == 1) return YGPU_OK;
    for (int it = 1; it <= maxiter; it++) {
        iters = it;
        __syncthreads();           // every thread has read the previous s_flag / s_sc[3]
        if (lead) {
            s_flag = (rho == W(0) || !isfinite(rho)) ? 2 : 0;
            s_sc[2] = (it == 1) ? W(0) : (rho / rho_old) * (alpha / omega);
            s_sc[1] = omega;
        }
        __syncthreads();
        if (s_flag == 2) { relres = (double)s_sc[3]; return YGPU_BREAKDOWN; }
        {
            const T beta = s_sc[2], om = s_sc[1];
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                T pu = (it == 1) ? r[u] : r[u] + beta * (p[u] - om * v[u]);
                p[u] = pu;
                if (!M) ph[u] = precond ? (T)dinv[u] * pu : pu;
            }
        }
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
        // ILU(0): p_hat = M^-1 p over every row (barriers inside)
        if (M && !(ok = ilu_apply<T>(Tm, M->nx, M->n2, nu, M->icol, M->lu, M->pivinv, p, ph))) return YGPU_ERR_TIMEOUT;
        A.apply(Tm, ph, v, R);
        T tvp = T(0);
        {
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                tvp += rt[u] * v[u];
            }
        }
        T tv = T(0);
        if (!(ok = team_allreduce_w<T>(Tm, &tvp, &tv, 1))) return YGPU_ERR_TIMEOUT;
        if (lead) {
            if (tv == T(0) || !isfinite(tv)) s_flag = 2;
            else {
                alpha = rho / tv;
                s_sc[0] = alpha;
                s_flag = 0;
            }
        }
        __syncthreads();
        if (s_flag == 2) { relres = (double)s_sc[3]; return YGPU_BREAKDOWN; }
        const T al = s_sc[0];
        T ssp = T(0);
        {
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                T su = r[u] - al * v[u];
                s[u] = su;
                if (!M) sh[u] = precond ? (T)dinv[u] * su : su;
                ssp += su * su;
            }
        }
        // ||s|| rides on the next all-reduce: t = A sh is computed before the
        // early-convergence test on s, which saves an all-reduce per iteration
        // (the last iteration's t is then unused)
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
        if (M && !(ok = ilu_apply<T>(Tm, M->nx, M->n2, nu, M->icol, M->lu, M->pivinv, s, sh))) return YGPU_ERR_TIMEOUT;
        A.apply(Tm, sh, t, R);
        T ts0 = T(0), ts1 = T(0);
        {
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                const T tu = t[u];
                ts0 += tu * s[u];
                ts1 += tu * tu;
            }
        }
        T ts[3];
        {
            const T part[3] = {ts0, ts1, ssp};
            if (!(ok = team_allreduce_w<T>(Tm, part, ts, 3))) return YGPU_ERR_TIMEOUT;
        }
        if (lead) {
            s_sc[3] = sqrt(ts[2]) / (W)bnrm;
            if (s_sc[3] <= (W)tol) s_flag = 1;
            else if (ts[1] == T(0) || !isfinite(ts[1])) s_flag = 2;
            else {
                omega = ts[0] / ts[1];
                s_sc[1] = omega;
                s_flag = 0;
            }
        }
        __syncthreads();
        if (s_flag == 1) {
            relres = (double)s_sc[3];
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                x[u] = x[u] + al * ph[u];
            }
            if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
            return YGPU_OK;
        }
        if (s_flag == 2) { relres = (double)s_sc[3]; return YGPU_BREAKDOWN; }
        const T om = s_sc[1];
        T rr0 = T(0), rr1 = T(0);
        {
            int q = 0;
            for (int e = R.t0; e < R.t1; e += R.ts, q++) {
                const int u = R.row(e, q);
                x[u] = x[u] + al * ph[u] + om * sh[u];
                T ru = s[u] - om * t[u];
                r[u] = ru;
                rr0 += ru * ru;
                rr1 += rt[u] * ru;
            }
        }
        T rr[2];
        {
            const T part[2] = {rr0, rr1};
            if (!(ok = team_allreduce_w<T>(Tm, part, rr, 2))) return YGPU_ERR_TIMEOUT;
        }
        if (lead) {
            s_sc[3] = sqrt(rr[0]) / (W)bnrm;
            s_flag = (s_sc[3] <= (W)tol) ? 1 : ((omega == W(0)) ? 2 : 0);
            rho_old = rho;
            rho = rr[1];
        }
        __syncthreads();
        if (s_flag != 0) relres = (double)s_sc[3];
        if (s_flag == 1) return YGPU_OK;
        if (s_flag == 2) { relres = (double)s_sc[3]; return YGPU_BREAKDOWN; }
    }
    relres = (double)s_sc[3];
    return YGPU_MAXITER;
}

// ---------------------------------------------------------------------------
// Block preconditioner on C-grid tiles (the GPU form of LIS's -p ilu: block
// Jacobi, each block the exact inverse of a 4 x 4-cell tile of the operator)
//
// A tile holds the 32 unknowns of 16 cells; lane l of a warp owns unknown
// (cell l/2 of the tile, component l%2): cell (4 tx + (l/2)%4, 4 ty + l/8),
// ux for even l, uy for odd l. The tile block keeps the couplings of free rows
// to free columns inside the tile (Dirichlet, tied and out-of-grid rows are
// identity rows), so it is symmetric for the energy operator; Gauss-Jordan in
// registers (lane j holds column j) inverts it, and the inverse is stored
// column-major: minv[t*1024 + k*32 + l] = (block^-1)[l][k]. Applying it is a
// 32 x 32 matrix-vector product per warp through shuffles.
// ---------------------------------------------------------------------------
#define YG_TILE 4

YG_DEV int tile_count(const Geo& G) { return ((G.nx + YG_TILE - 1) / YG_TILE) * ((G.ny + YG_TILE - 1) / YG_TILE); }

// unknown of lane l in tile t, or -1 outside the grid
YG_DEV int tile_unknown(const Geo& G, int t, int l) {
    const int ntx = (G.nx + YG_TILE - 1) / YG_TILE;
    const int tx = t % ntx, ty = t / ntx;
    const int cl = l >> 1;
    const int i = tx * YG_TILE + (cl & 3), j = ty * YG_TILE + (cl >> 2);
    if (i >= G.nx || j >= G.ny) return -1;
    return ((l & 1) ? G.n2 : 0) + i + G.nx * j;
}

// lane of unknown u inside tile t, or -1 when u is in another tile
YG_DEV int tile_lane(const Geo& G, int t, int u) {
    const int pl = (u >= G.n2) ? 1 : 0;
    const int c = u - pl * G.n2;
    const int i = c % G.nx, j = c / G.nx;
    const int ntx = (G.nx + YG_TILE - 1) / YG_TILE;
    if ((i / YG_TILE) + ntx * (j / YG_TILE) != t) return -1;
    return 2 * ((i % YG_TILE) + YG_TILE * (j % YG_TILE)) + pl;
}

// coefficient of free column col in free row u outside the interior stencil
// (energy_row_general applied to the unit vector of col)
template <typename T, typename CT>
__device__ __noinline__ T energy_coef_general(const Inst& I, const Geo& G, const OpK<T>& K, const CT* N,
                                              const CT* Nab, const CT* dgx, const CT* dgy, int u, int col) {
    const int* emap = I.emap;
    auto unit = [&](int d) -> T { return (d >= 0 && emap[d] == col) ? T(1) : T(0); };
    const T vr = (u == col) ? T(1) : T(0);
    T acc = ((u < G.n2) ? (T)dgx[u] : (T)dgy[u - G.n2]) * vr;
    acc += member_elems<T>(G, K, N, Nab, u, unit);
    const int* mem = I.mem + 3 * u;
    for (int m = 0; m < 3; m++) {
        int mm = mem[m];
        if (mm < 0) break;
        acc += ((mm < G.n2) ? (T)dgx[mm] : (T)dgy[mm - G.n2]) * vr;
        acc += member_elems<T>(G, K, N, Nab, mm, unit);
    }
    return acc;
}

// Builds and inverts every tile block of the energy operator A (team-wide, one
// warp per tile). The row of each lane goes through the tile's inverse storage
// (row-major) to reach the lanes that hold the columns.
template <typename T, typename CT>
__device__ __noinline__ void block_setup(const Inst& I, const Geo& G, Team& Tm, const StencilOp<T, CT>& A, T* minv) {
    const int lane = threadIdx.x & 31;
    const int gw = Tm.tid >> 5, nw = Tm.nthr >> 5;
    const int nt = tile_count(G);
    const int nx = G.nx, ny = G.ny, n2 = G.n2;
    for (int t = gw; t < nt; t += nw) {
        T* M = minv + (size_t)t * 1024;
        const int u = tile_unknown(G, t, lane);
        // row of this lane: zero, then its in-tile couplings
        for (int k = 0; k < 32; k++) M[lane * 32 + k] = T(0);
        if (u < 0 || I.ukind[u] != DOF_FREE) {
            M[lane * 32 + lane] = T(1);
        } else {
            const int pl = (u >= n2) ? 1 : 0;
            const int c = u - pl * n2;
            const int i = c % nx, j = c / nx;
            const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
            const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
            // the nine columns of the row's stencil and, on the interior stencil, their coefficients
            int col[9];
            T cf[9];
            const bool fast = (I.rpart[u] == 1);
            const T dyodx = A.K.dyodx, dxody = A.K.dxody;
            if (pl == 0) {
                col[0] = c; col[1] = ip1 + nx * j; col[2] = im1 + nx * j; col[3] = i + nx * jp1; col[4] = i + nx * jm1;
                col[5] = n2 + c; col[6] = n2 + ip1 + nx * j; col[7] = n2 + ip1 + nx * jm1; col[8] = n2 + i + nx * jm1;
                if (fast) {
                    const T Ni = (T)A.N[c], Np = (T)A.N[ip1 + nx * j], Bc = (T)A.Nab[c], Bm = (T)A.Nab[i + nx * jm1];
                    cf[0] = T(4) * dyodx * (Np + Ni) + dxody * (Bc + Bm) + (T)A.dgx[c];
                    cf[1] = -T(4) * dyodx * Np; cf[2] = -T(4) * dyodx * Ni;
                    cf[3] = -dxody * Bc; cf[4] = -dxody * Bm;
                    cf[5] = T(2) * Ni + Bc; cf[6] = -(T(2) * Np + Bc); cf[7] = T(2) * Np + Bm; cf[8] = -(T(2) * Ni + Bm);
                }
            } else {
                col[0] = u; col[1] = n2 + i + nx * jp1; col[2] = n2 + i + nx * jm1; col[3] = n2 + ip1 + nx * j;
                col[4] = n2 + im1 + nx * j;
                col[5] = c; col[6] = i + nx * jp1; col[7] = im1 + nx * jp1; col[8] = im1 + nx * j;
                if (fast) {
                    const T Ni = (T)A.N[c], Np = (T)A.N[i + nx * jp1], Bc = (T)A.Nab[c], Bm = (T)A.Nab[im1 + nx * j];
                    cf[0] = T(4) * dxody * (Np + Ni) + dyodx * (Bc + Bm) + (T)A.dgy[c];
                    cf[1] = -T(4) * dxody * Np; cf[2] = -T(4) * dxody * Ni;
                    cf[3] = -dyodx * Bc; cf[4] = -dyodx * Bm;
                    cf[5] = T(2) * Ni + Bc; cf[6] = -(T(2) * Np + Bc); cf[7] = T(2) * Np + Bm; cf[8] = -(T(2) * Ni + Bm);
                }
            }
#pragma unroll 1
            for (int q = 0; q < 9; q++) {
                const int cu = col[q];
                const int cl = tile_lane(G, t, cu);
                if (cl < 0 || I.ukind[cu] != DOF_FREE) continue;
                const T v = fast ? cf[q] : energy_coef_general<T, CT>(I, G, A.K, A.N, A.Nab, A.dgx, A.dgy, u, cu);
                M[lane * 32 + cl] += v;
            }
        }
        __syncwarp();
        // symmetric diagonal scaling S B S (S = |diag|^-1/2) before the FP32
        // inversion: the viscosity contrast of the ice makes the raw blocks far
        // worse conditioned than the scaled ones
        const T dl = M[lane * 32 + lane];
        const T sl = (dl > T(0) && isfinite(dl)) ? T(1) / sqrt(dl) : T(1);
        // lane j takes column j of the scaled block, and column j of the identity
        T a[32], x[32];
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const T sr = __shfl_sync(0xffffffffu, sl, r);
            a[r] = sr * M[r * 32 + lane] * sl;
            x[r] = (r == lane) ? T(1) : T(0);
        }
        __syncwarp();
        // Gauss-Jordan without pivoting (symmetric positive definite blocks). A
        // pivot below 1e-5 of its original diagonal (a tile block that is
        // singular on its own, e.g. a floating tile without basal drag, whose
        // rigid translations have no energy inside the tile) or a non-finite one
        // turns the whole tile into Jacobi.
        const T d0 = a[lane];
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 32; k++) {
            const T p = __shfl_sync(0xffffffffu, a[k], k);
            const T dk = __shfl_sync(0xffffffffu, d0, k);
            if (!(p > T(1e-5) * fabs(dk)) || !isfinite(p)) bad = true;
            const T ip = bad ? T(0) : T(1) / p;
            a[k] *= ip;
            x[k] *= ip;
#pragma unroll
            for (int r = 0; r < 32; r++) {
                if (r == k) continue;
                const T f = __shfl_sync(0xffffffffu, a[r], k);     // A[r][k]
                a[r] -= f * a[k];
                x[r] -= f * x[k];
            }
        }
        bad = __any_sync(0xffffffffu, bad);
        if (bad) {
#pragma unroll
            for (int r = 0; r < 32; r++) x[r] = T(0);
            x[lane] = T(1);       // unscaled below: 1/d, or 1 where the diagonal is not positive
        }
        // column `lane` of the inverse S (SBS)^-1 S, column-major: element
        // (r, lane) at lane * 32 + r
#pragma unroll
        for (int r = 0; r < 32; r++) {
            const T sr = __shfl_sync(0xffffffffu, sl, r);
            M[lane * 32 + r] = sr * x[r] * sl;
        }
        __syncwarp();
    }
}

// out = M^-1 in for the whole team (tile mapping; the caller separates it from
// row-mapped loops by team barriers)
template <typename T, typename MT>
YG_DEV T block_apply_lane(const MT* M, T w, int lane) {
    T acc = T(0);
#pragma unroll
    for (int k = 0; k < 32; k++) acc += (T)M[k * 32 + lane] * __shfl_sync(0xffffffffu, w, k);
    return acc;
}

// Pipelined CG (as krylov_pcg_pipe) with the tile-block preconditioner: every
// loop runs over tiles, one warp per tile and one unknown per lane, so the
// preconditioner is applied to a tile's freshly computed vector through warp
// shuffles in the same pass.
template <typename T, typename Op>
__device__ __noinline__ int krylov_pcg_pipe_blk(Team& Tm_, const Geo& G, const Op& A, const float* __restrict__ minv,
                                                T* __restrict__ x, const T* __restrict__ b, T* __restrict__ r,
                                                T* __restrict__ u, T* __restrict__ w, T* m0, T* m1, T* __restrict__ z,
                                                T* __restrict__ q, T* __restrict__ s, T* __restrict__ p, int maxiter,
                                                double tol, double bnrm, int& iters, double& relres, bool& ok) {
    TeamLocal tl_(Tm_);
    Team& Tm = tl_.t;
    __shared__ T s_ab[3];          // alpha, beta, relres (in T, as in krylov_pcg_pipe)
    __shared__ int s_flag;
    const bool lead = (threadIdx.x == 0);
    using W = T;                   // precision of the scalar recurrences
    const int lane = threadIdx.x & 31, gw = Tm.tid >> 5, nw = Tm.nthr >> 5, nt = tile_count(G);
    ok = true;
    iters = 0;
    int it = 0;
    for (int restart = 0; restart < 8; restart++) {
        // r = b - A x, u = M r
        for (int t = gw; t < nt; t += nw) {
            const int k = tile_unknown(G, t, lane);
            const T rk = (k >= 0) ? b[k] - A.row(k, x) : T(0);
            const T uk = block_apply_lane(minv + (size_t)t * 1024, rk, lane);
            if (k >= 0) { r[k] = rk; u[k] = uk; }
        }
        if (!(ok = team_barrier(Tm))) return YGPU_ERR_TIMEOUT;
        // w = A u, m = M w, partial dots
        T a0 = T(0), a1 = T(0), a2 = T(0);
        for (int t = gw; t < nt; t += nw) {
            const int k = tile_unknown(G, t, lane);
            const T wk = (k >= 0) ? A.row(k, u) : T(0);
            const T mk = block_apply_lane(minv + (size_t)t * 1024, wk, lane);
            if (k >= 0) {
                w[k] = wk;
                m0[k] = mk;
                z[k] = T(0); q[k] = T(0); s[k] = T(0); p[k] = T(0);
                const T rk = r[k], uk = u[k];
                a0 += rk * uk;
                a1 += wk * uk;
                a2 += rk * rk;
            }
        }
        T red[3];
        {
            const T part[3] = {a0, a1, a2};
            if (!(ok = team_allreduce_w<T>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
        }
        W gam_old = W(1), alpha_old = W(1);
        if (lead) {
            const W rel = sqrt(red[2]) / (W)bnrm;
            s_ab[2] = rel;
            if (rel <= (W)tol) s_flag = 1;
            else {
                const W gam = red[0], del = red[1];
                const W alpha = gam / del;
                if (!isfinite(alpha) || del == W(0)) s_flag = 2;
                else {
                    s_flag = 0;
                    s_ab[0] = alpha;
                    s_ab[1] = W(0);
                    gam_old = gam;
                    alpha_old = alpha;
                }
            }
        }
        __syncthreads();
        if (s_flag == 1) { relres = (double)s_ab[2]; iters = it; return YGPU_OK; }
        if (s_flag == 2) { relres = (double)s_ab[2]; iters = it; return (it < maxiter) ? YGPU_BREAKDOWN : YGPU_MAXITER; }
        T* mc = m0;
        T* mn = m1;
        bool recheck = false;
        while (it < maxiter) {
            const T a = s_ab[0], bt = s_ab[1];
            a0 = a1 = a2 = T(0);
            for (int t = gw; t < nt; t += nw) {
                const int k = tile_unknown(G, t, lane);
                T wk = T(0);
                if (k >= 0) {
                    const T nk = A.row(k, mc);
                    const T zk = nk + bt * z[k];
                    const T qk = mc[k] + bt * q[k];
                    const T sk = w[k] + bt * s[k];
                    const T pk = u[k] + bt * p[k];
                    z[k] = zk; q[k] = qk; s[k] = sk; p[k] = pk;
                    x[k] = x[k] + a * pk;
                    const T rk = r[k] - a * sk;
                    const T uk = u[k] - a * qk;
                    wk = w[k] - a * zk;
                    r[k] = rk; u[k] = uk; w[k] = wk;
                    a0 += rk * uk;
                    a1 += wk * uk;
                    a2 += rk * rk;
                }
                const T mk = block_apply_lane(minv + (size_t)t * 1024, wk, lane);
                if (k >= 0) mn[k] = mk;
            }
            it++;
            {
                const T part[3] = {a0, a1, a2};
                if (!(ok = team_allreduce_w<T>(Tm, part, red, 3))) return YGPU_ERR_TIMEOUT;
            }
            { T* tt = mc; mc = mn; mn = tt; }
            if (lead) {
                // FP32 inner solves: the recurrence scalars in FP32 (its division
                // and square root are far faster than FP64's on this part)
                const W rel = sqrt(red[2]) / (W)bnrm;
                s_ab[2] = rel;
                if (!isfinite(rel)) s_flag = 2;
                else if (rel <= (W)tol) s_flag = 1;
                else {
                    const W gam = red[0], del = red[1];
                    const W beta = gam / gam_old;
                    const W alpha = gam / (del - beta * gam / alpha_old);
                    if (!isfinite(alpha) || !isfinite(beta) || del == W(0)) s_flag = 3;
                    else {
                        s_flag = 0;
                        s_ab[0] = alpha;
                        s_ab[1] = beta;
                        gam_old = gam;
                        alpha_old = alpha;
                    }
                }
            }
            __syncthreads();
            const int flag = s_flag;
            if (flag != 0) relres = (double)s_ab[2];
            if (flag == 2) { iters = it; return YGPU_BREAKDOWN; }
            if (flag == 1) { recheck = true; break; }
            if (flag == 3) {
                if (it < maxiter) { iters = it; return YGPU_BREAKDOWN; }
                break;
            }
        }
        iters = it;
        relres = (double)s_ab[2];
        if (!recheck) return YGPU_MAXITER;
        T tr = T(0);
        for (int k = Tm.tid; k < G.nu; k += Tm.nthr) {
            const T rk = b[k] - A.row(k, x);
            tr += rk * rk;
        }
        {
            T trs;
            if (!(ok = team_allreduce_w<T>(Tm, &tr, &trs, 1))) return YGPU_ERR_TIMEOUT;
            tr = trs;
        }
        relres = (double)(sqrt(tr) / (W)bnrm);
        if (relres <= tol) return YGPU_OK;
        if (it >= maxiter) return YGPU_MAXITER;
    }
    return YGPU_MAXITER;
}

// ---------------------------------------------------------------------------
// Linear solve of one Picard iteration: FP64, or FP32 inside FP64 defect correction
// ---------------------------------------------------------------------------
__device__ __noinline__ int linear_solve(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T, double bnrm, int& iters,
                        double& relres, int& outer, bool& ok) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool energy = (P.ssa_solver == YGPU_SSA_ENERGY);
    const bool pre = (P.lin_precond != YGPU_PRE_NONE);
    // MINRES requests run CG on the symmetric energy system, BiCGSTAB on the residual one
    const bool use_cg = energy ? (P.lin_solver != YGPU_LIN_BICGSTAB) : false;
    outer = 0;
    const StencilOp<double, double> A64{&I, &G, energy, I.visc_int, I.Nab, I.drag_x, I.drag_y, make_opk<double>(G),
                                        I.acell};
    if (P.precision != YGPU_PREC_MIXED || krylov_fp64_ilu(I, P, G)) {
        // -p ilu on the energy form: the FP32 tile inverses (built by the pre step)
        // precondition the FP64 CG
        if (use_cg && energy && P.lin_precond == YGPU_PRE_ILU0 && I.fminv)
            return krylov_pcg_pipe_blk<double>(T, G, A64, I.fminv, I.x, I.b, I.r, I.rt, I.v, I.ph, I.m2, I.z, I.q,
                                               I.s, I.p, P.lin_maxiter, P.lin_tol, bnrm, iters, relres, ok);
        if (use_cg)
            return krylov_pcg_pipe<double>(T, G.nu, A64, I.dinv, I.x, I.b, I.r, I.rt, I.v, I.ph, I.m2, I.z, I.q, I.s,
                                           I.p, P.lin_maxiter, P.lin_tol, bnrm, pre, iters, relres, ok);
        if (!energy && I.icol && I.ilu && ilu_colourable(G)) {
            const IluM<double> M{G.nx, G.n2, I.icol, I.ilu, I.ipiv};
            return krylov_bicgstab<double>(T, G.nu, A64, I.dinv, I.x, I.b, I.r, I.rt, I.p, I.v, I.s, I.t, I.ph, I.sh,
                                           P.lin_maxiter, P.lin_tol, bnrm, pre, iters, relres, ok, &M);
        }
        return krylov_bicgstab<double>(T, G.nu, A64, I.dinv, I.x, I.b, I.r, I.rt, I.p, I.v, I.s, I.t, I.ph, I.sh,
                                       P.lin_maxiter, P.lin_tol, bnrm, pre, iters, relres, ok);
    }
    const StencilOp<float, float> A32{&I, &G, energy, I.fN, I.fNab, I.fdrag_x, I.fdrag_y, make_opk<float>(G),
                                      I.acell};
    // ---- mixed: FP32 coefficients (copied by the pre step, with the tile-block
    // inverses of -p ilu), FP32 inner Krylov, FP64 outer residual ----
    const bool block = use_cg && energy && P.lin_precond == YGPU_PRE_ILU0 && I.fminv;
    const double inner_tol = (P.inner_tol > 0.0) ? P.inner_tol : 1e-3;
    // inner solves are capped: one that cannot reach inner_tol in FP32 (an
    // operator too ill-conditioned for single precision) still hands its
    // progress to the FP64 defect correction instead of running to lin_maxiter
    const int inner_max = (P.inner_maxiter > 0) ? P.inner_maxiter : (P.lin_maxiter < 400 ? P.lin_maxiter : 400);
    int total = 0;
    int status = YGPU_MAXITER;
    const int max_outer = 200;           // total inner iterations stay below lin_maxiter
    // The outer passes visit the rows of the active cells only (identity rows
    // hold x = b, a zero residual and a zero correction, cleared here once).
    const RowItems R = make_row_items(T, I.acell, G.n2, G.nu, false);
    // the FP32 cell CG reads the FP64 residual on every row (zero outside the
    // active rows since the setup step) and adds its correction to x itself;
    // the other inner solvers take FP32 copies
    const bool cells = use_cg && !block && I.fst && G.nx <= (1 << 14) && G.ny <= (1 << 14);
    for (int u = t_tid; u < G.nu; u += t_nthr) {
        I.fr[u] = 0.0f;
        I.fx[u] = 0.0f;
    }
    for (int o = 0; o < max_outer; o++) {
        // r64 = b - A64 x (FP64 residual of the outer iterate)
        A64.apply(T, I.x, I.q, R);
        double rr = 0.0;
        for (int e = R.t0; e < R.t1; e += R.ts) {
            const int u = R.lookup(e);
            double ru = I.b[u] - I.q[u];
            I.r[u] = ru;
            rr += ru * ru;
        }
        if (!(ok = team_allreduce(T, &rr, 1))) return YGPU_ERR_TIMEOUT;
        relres = sqrt(rr) / bnrm;
        if (relres <= P.lin_tol) { status = YGPU_OK; break; }
        // a non-finite residual (non-finite coefficients or right-hand side) ends the
        // solve as the FP64 Krylov methods do, before a correction scaled by it
        if (!isfinite(relres)) { status = YGPU_BREAKDOWN; break; }
        if (total >= P.lin_maxiter) { status = YGPU_MAXITER; break; }
        // inner FP32 solve of A d = r, d0 = 0, scaled by ||r||
        const double nr = sqrt(rr), sc = 1.0 / nr;
        int it = 0;
        double rel_in = 0.0;
        int st;
        if (cells) {
            st = krylov_pcg_cells(T, G.nu, A32, I.fdinv, I.x, nr, I.r, sc, I.fv, I.fph, I.fm2, I.fst, inner_max,
                                  inner_tol, pre, it, rel_in, ok);
            if (!ok) return YGPU_ERR_TIMEOUT;
            total += it;
            outer++;
            if (st == YGPU_BREAKDOWN && it <= 1) { status = YGPU_BREAKDOWN; break; }
            continue;
        }
        for (int e = R.t0; e < R.t1; e += R.ts) {
            const int u = R.lookup(e);
            I.fr[u] = (float)(I.r[u] * sc);
            I.fx[u] = 0.0f;
        }
        if (!(ok = team_barrier(T))) return YGPU_ERR_TIMEOUT;
        if (use_cg && block)
            st = krylov_pcg_pipe_blk<float>(T, G, A32, I.fminv, I.fx, I.fr, I.frt, I.fv, I.ft, I.fph, I.fm2, I.fz,
                                            I.fq, I.fs, I.fp, inner_max, inner_tol, 1.0, it, rel_in, ok);
        else if (use_cg)
            st = krylov_pcg_pipe<float>(T, G.nu, A32, I.fdinv, I.fx, I.fr, I.frt, I.fv, I.ft, I.fph, I.fm2, I.fz,
                                        I.fq, I.fs, I.fp, inner_max, inner_tol, 1.0, pre, it, rel_in, ok);
        else
            st = krylov_bicgstab<float>(T, G.nu, A32, I.fdinv, I.fx, I.fr, I.fz, I.frt, I.fp, I.fv, I.fs, I.ft, I.fph,
                                        I.fsh, inner_max, inner_tol, 1.0, pre, it, rel_in, ok);
        if (!ok) return YGPU_ERR_TIMEOUT;
        total += it;
        outer++;
        // x += d (FP64 accumulation)
        for (int e = R.t0; e < R.t1; e += R.ts) {
            const int u = R.lookup(e);
            I.x[u] = I.x[u] + (double)I.fx[u] * nr;
        }
        if (!(ok = team_barrier(T))) return YGPU_ERR_TIMEOUT;
        if (st == YGPU_BREAKDOWN && it <= 1) { status = YGPU_BREAKDOWN; break; }
    }
    iters = total;
    return status;
}

// ---------------------------------------------------------------------------
// Phase: epilogue of one Picard iteration
// ---------------------------------------------------------------------------
// Magnitude tests of a double on the integer pipe: the magnitude bits order
// like the absolute value, with inf above every finite bound and NaN above inf.
// b is a positive finite bound.
YG_DEV unsigned long long dmag(double v) { return (unsigned long long)__double_as_longlong(v) & 0x7fffffffffffffffull; }
YG_DEV unsigned long long dbits(double b) { return (unsigned long long)__double_as_longlong(b); }
// fabs(v) < b (false for NaN)
YG_DEV bool abs_lt(double v, double b) { return dmag(v) < dbits(b); }
// fabs(v) > b (false for NaN)
YG_DEV bool abs_gt(double v, double b) { const unsigned long long m = dmag(v); return m > dbits(b) && m <= 0x7ff0000000000000ull; }
YG_DEV bool finite_d(double v) { return dmag(v) < 0x7ff0000000000000ull; }

__device__ __noinline__ void phase_epilogue(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T, bool diva, double red[4]) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool energy = (P.ssa_solver == YGPU_SSA_ENERGY);
    const double lim = P.ssa_vel_max, rel = P.ssa_iter_rel;
    const double vel_tol = 1e-5;
    // the tests and counts on the integer pipe (GB300's FP64 pipe is slow): the
    // FP64 work left is the relaxation, the norm sums and the basal terms
    double r1 = 0.0, r2 = 0.0;
    int nchk = 0, nbad = 0;
    for (int c = t_tid; c < G.n2; c += t_nthr) {
        double uv[2];
#pragma unroll
        for (int pl = 0; pl < 2; pl++) {
            const int u = pl * G.n2 + c;
            int src = u;
            if (energy) {
                int e = I.emap[u];
                if (e >= 0) src = e;
            }
            double val = I.x[src];
            // linear_solver_save_velocity: underflow flush
            if (abs_lt(val, TOL_UNDERFLOW)) val = 0.0;
            // ssa_vel_clip (NaN passes through)
            if (abs_gt(val, lim)) val = copysign(lim, val);
            // picard_relax_vel
            const double up = pl ? I.uy_nm1[c] : I.ux_nm1[c];
            val = up + rel * (val - up);
            uv[pl] = val;
            // picard_calc_convergence_l2 contributions
            const int mask = pl ? I.mask_y[c] : I.mask_x[c];
            if (abs_gt(val, vel_tol) && mask > 0) {
                nchk++;
                double t = val - up;
                if (abs_lt(t, TOL_UNDERFLOW)) t = 0.0;
                r1 += t * t;
                t = up;
                if (abs_lt(t, TOL_UNDERFLOW)) t = 0.0;
                r2 += t * t;
            }
            if (mask > 0 && !finite_d(val)) nbad++;
        }
        I.u_x[c] = uv[0];
        I.u_y[c] = uv[1];
        if (diva) {
            // calc_basal_stress (velocity_diva.f90:1011-1050) and calc_vel_basal (:960-1009)
            double tx = I.bm_x[c] * uv[0];
            if (abs_lt(tx, TOL_UNDERFLOW)) tx = 0.0;
            double ty = I.bm_y[c] * uv[1];
            if (abs_lt(ty, TOL_UNDERFLOW)) ty = 0.0;
            I.taub_x[c] = tx;
            I.taub_y[c] = ty;
            if (P.no_slip) {
                I.ux_b[c] = 0.0;
                I.uy_b[c] = 0.0;
            } else {
                I.ux_b[c] = uv[0] - tx * I.F2x[c];
                I.uy_b[c] = uv[1] - ty * I.F2y[c];
            }
        }
    }
    red[0] = r1;
    red[1] = r2;
    red[2] = (double)nchk;
    red[3] = (double)nbad;
}

// picard_calc_convergence_l1rel_matrix of the last iteration (an output only):
// from the relaxed velocity and the previous iterate, once the loop finishes
__device__ __noinline__ void phase_err(const Inst& I, const Geo& G, Team& T) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    for (int c = t_tid; c < G.n2; c += t_nthr) {
#pragma unroll
        for (int pl = 0; pl < 2; pl++) {
            const double val = pl ? I.u_y[c] : I.u_x[c];
            const double up = pl ? I.uy_nm1[c] : I.ux_nm1[c];
            const double err = (fabs(val) > 1e-2) ? 2.0 * fabs(val - up) / fabs(val + up + 1e-5) : 0.0;
            if (pl) I.err_y[c] = err; else I.err_x[c] = err;
        }
    }
}

// ---------------------------------------------------------------------------
// Final passes after the Picard loop
// ---------------------------------------------------------------------------
__device__ __noinline__ double count_lim_part(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool drag = (P.ssa_vel_lim_method == YGPU_VEL_LIM_DRAG);
    const double s0 = 0.8 * P.ssa_vel_max, umax = P.ssa_vel_max;
    const double* ux = I.u_x;
    const double* uy = I.u_y;
    double n = 0.0;
    for (int c = t_tid; c < G.n2; c += t_nthr) {
        Nb b = make_nb(G, c);
        const int i = b.i, j = b.j;
        if (I.mask_x[c] >= 1) {
            if (drag) {
                double uc = 0.25 * (uy[c] + uy[CI(b.ip1, j)] + uy[CI(i, b.jm1)] + uy[CI(b.ip1, b.jm1)]);
                if (ux[c] * ux[c] + uc * uc > s0 * s0) n += 1.0;
            } else if (fabs(ux[c]) >= umax) n += 1.0;
        }
        if (I.mask_y[c] >= 1) {
            if (drag) {
                double uc = 0.25 * (ux[c] + ux[CI(b.im1, j)] + ux[CI(i, b.jp1)] + ux[CI(b.im1, b.jp1)]);
                if (uy[c] * uy[c] + uc * uc > s0 * s0) n += 1.0;
            } else if (fabs(uy[c]) >= umax) n += 1.0;
        }
    }
    return n;
}

// DIVA: final vertical shear (from the state at the start of the last
// iteration) and the 3D velocity (calc_vel_horizontal_3D, velocity_diva.f90:431-508)
__device__ __noinline__ void phase_diva_final(const Inst& I, const Geo& G, Team& T, const double* vlast_cur, const double* vfinal) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const int n2 = G.n2, nz = G.nz;
    const double* f = I.f_ice;
    const double* zeta = I.zeta;
    for (int c = t_tid; c < n2; c += t_nthr) {
        Nb n = make_nb(G, c);
        const int cx = CI(n.ip1, n.j), cy = CI(n.i, n.jp1);
        double F1c = 0.0, F1x = 0.0, F1y = 0.0;
        double gc = 0.0, gx = 0.0, gy = 0.0;
        const bool ic = (f[c] == 1.0), ix = (f[cx] == 1.0), iy = (f[cy] == 1.0);
        for (int k = 0; k < nz; k++) {
            const size_t o = (size_t)k * n2;
            const double omz = 1.0 - zeta[k];
            // F1 up to level k at this cell and its +x / +y neighbours
            double g0 = ic ? (I.H[c] / vfinal[o + c]) * omz : 0.0;
            double g1 = ix ? (I.H[cx] / vfinal[o + cx]) * omz : 0.0;
            double g2 = iy ? (I.H[cy] / vfinal[o + cy]) * omz : 0.0;
            if (k > 0) {
                const double dz = zeta[k] - zeta[k - 1];
                F1c = F1c + 0.5 * (g0 + gc) * dz;
                F1x = F1x + 0.5 * (g1 + gx) * dz;
                F1y = F1y + 0.5 * (g2 + gy) * dz;
            }
            gc = g0; gx = g1; gy = g2;
            double fa = stag_margin(ic ? F1c : 0.0, ix ? F1x : 0.0, f[c], f[cx]);
            double ux = I.ux_b[c] + I.taub_x[c] * fa;
            fa = stag_margin(ic ? F1c : 0.0, iy ? F1y : 0.0, f[c], f[cy]);
            double uy = I.uy_b[c] + I.taub_y[c] * fa;
            I.ux3[o + c] = ux;
            I.uy3[o + c] = uy;
            I.ux_i[o + c] = ux - I.ux_b[c];
            I.uy_i[o + c] = uy - I.uy_b[c];
        }
    }
}

// ---------------------------------------------------------------------------
// The Picard loop as steps: setup / pre (strain, shear, column, faces,
// system) / krylov / post (epilogue, convergence, final passes). Each step
// is a cooperative kernel over teams of CTAs; the state between steps lives
// in the instance's InstOut. The heavy steps and the lean Krylov kernel have
// their own register budgets and block sizes.
// ---------------------------------------------------------------------------
struct PhaseClock {
    unsigned long long t0;
    YG_DEV void start() { t0 = global_ns(); }
    YG_DEV double lap() {
        unsigned long long t = global_ns();
        double d = (double)(t - t0);
        t0 = t;
        return d;
    }
};

__device__ __noinline__ void step_setup(const Inst& I, const ygpu_dyn_par& P, Team& T, int* done_count) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const bool diva = (I.kind == YGPU_KIND_DIVA);
    const Geo G = make_geo(I, P);
    InstOut* out = I.out;
    const bool lead = (T.cta == 0 && threadIdx.x == 0);
    PhaseClock clk;
    clk.start();
    for (int c = t_tid; c < G.n2; c += t_nthr) {
        I.err_x[c] = 1.0;
        I.err_y[c] = 1.0;
        I.cflag[c] = cell_flags(G, I, c);
        // the mixed defect correction writes its FP64 residual on the active
        // rows only; the FP32 cell CG reads it on every row
        if (P.precision == YGPU_PREC_MIXED) {
            I.r[c] = 0.0;
            I.r[G.n2 + c] = 0.0;
        }
        if (!diva) {
            // set_inactive_margins (velocity_general.f90:1687-1750), SSA only
            Nb n = make_nb(G, c);
            const double fa = I.f_ice[c];
            double fb = I.f_ice[CI(n.ip1, n.j)];
            if ((fb == 0.0 && fa < 1.0) || (fa == 0.0 && fb < 1.0)) I.u_x[c] = 0.0;
            fb = I.f_ice[CI(n.i, n.jp1)];
            if ((fb == 0.0 && fa < 1.0) || (fa == 0.0 && fb < 1.0)) I.u_y[c] = 0.0;
        }
    }
    int status = YGPU_OK;
    if (!team_barrier(T)) status = YGPU_ERR_TIMEOUT;
    else if (!phase_classify(I, P, G, T)) status = ld_acquire_s32(T.abort_all) ? YGPU_ERR_TIMEOUT : YGPU_ERR_BAD_ARG;
    else {
        if (P.visc_method != 0) phase_att_powers(I, P, G, T);
        if (!team_barrier(T)) status = YGPU_ERR_TIMEOUT;
    }
    if (lead) {
        out->phase_ns[0] += clk.lap();
        out->status = status;
        out->done = (status != YGPU_OK);
        if (status != YGPU_OK) atomicAdd(done_count, 1);
    }
}

__device__ __noinline__ void step_pre(const Inst& I, const ygpu_dyn_par& P, Team& T, int* done_count) {
    const bool diva = (I.kind == YGPU_KIND_DIVA);
    const Geo G = make_geo(I, P);
    InstOut* out = I.out;
    const bool lead = (T.cta == 0 && threadIdx.x == 0);
    double* sdudx = I.lk_x;
    double* sdudy = I.lk_y;
    double* sdvdx = I.lr_x;
    double* sdvdy = I.lr_y;
    const int iter = out->iter_now + 1;
    const int in_alt = out->in_alt;
    double* vcur = in_alt ? I.visc_alt : I.visc;
    double* vnew = in_alt ? I.visc : I.visc_alt;
    // mixed mode: FP32 working copies of the viscosity in the visc_alt storage
    // (current one: vf[in_alt] from the second iteration on; the first reads
    // the caller's FP64 viscosity)
    const bool mixed = (P.precision == YGPU_PREC_MIXED);
    float* vf0 = (float*)I.visc_alt;
    float* vf1 = vf0 + (size_t)G.n2 * G.nz;
    const float* vcur_f = in_alt ? vf1 : vf0;
    float* vnew_f = in_alt ? vf0 : vf1;
    const bool relax = diva ? true : (P.visc_method != 0);
    PhaseClock clk;
    clk.start();
    double t1 = 0, t2 = 0, t3 = 0, t4 = 0;
    int status = YGPU_OK;
    double bn2 = 0.0;
    // mixed mode: the strain rates in FP32 (the column pass computes in FP32),
    // stored in the first half of the same scratch arrays
    float* fsdudx = (float*)sdudx;
    float* fsdudy = (float*)sdudy;
    float* fsdvdx = (float*)sdvdx;
    float* fsdvdy = (float*)sdvdy;
    if (P.visc_method == 1 || diva) {
        if (P.visc_method == 1) {
            if (mixed) phase_strain<float>(I, G, T, I.u_x, I.u_y, fsdudx, fsdudy, fsdvdx, fsdvdy);
            else phase_strain<double>(I, G, T, I.u_x, I.u_y, sdudx, sdudy, sdvdx, sdvdy);
        }
        if (diva) {
            if (!mixed) phase_shear<double, double>(I, G, T, vcur);
            else if (iter == 1) phase_shear<float, double>(I, G, T, I.visc);
            else phase_shear<float, float>(I, G, T, vcur_f);
        }
        if (!team_barrier(T)) { status = YGPU_ERR_TIMEOUT; goto out_; }
    }
    t1 = clk.lap();
    if (mixed)
        phase_column<float, float, float>(I, P, G, T, I.visc, vnew_f, fsdudx, fsdudy, fsdvdx, fsdvdy, relax, diva, true,
                                          iter > 1);
    else
        phase_column<double, double>(I, P, G, T, vcur, vnew, sdudx, sdudy, sdvdx, sdvdy, relax, diva, true, iter > 1);
    if (!team_barrier(T)) { status = YGPU_ERR_TIMEOUT; goto out_; }
    t2 = clk.lap();
    if (mixed) phase_faces<float>(I, P, G, T, diva);
    else phase_faces<double>(I, P, G, T, diva);
    if (!team_barrier(T)) { status = YGPU_ERR_TIMEOUT; goto out_; }
    t3 = clk.lap();
    phase_system(I, P, G, T, bn2);
    if (!team_allreduce(T, &bn2, 1)) { status = YGPU_ERR_TIMEOUT; goto out_; }
    if (!mixed && I.fminv && P.ssa_solver == YGPU_SSA_ENERGY && P.lin_precond == YGPU_PRE_ILU0) {
        // FP64 solve with -p ilu: FP32 tile inverses from the FP64 coefficients
        const StencilOp<float, double> Ab{&I, &G, true, I.visc_int, I.Nab, I.drag_x, I.drag_y, make_opk<float>(G)};
        block_setup<float, double>(I, G, T, Ab, I.fminv);
        if (!team_barrier(T)) { status = YGPU_ERR_TIMEOUT; goto out_; }
    }
    if (I.icol && P.ssa_solver != YGPU_SSA_ENERGY && ilu_colourable(G)) {
        // -p ilu on the residual form: the FP64 ILU(0) factors of this iteration's
        // operator (the mixed mode's coefficients are its FP32 values widened)
        const bool okf = ilu_factor<double, double>(I, G, T, I.visc_int, I.Nab, I.drag_x, I.drag_y, I.ilu, I.ipiv);
        if (!okf) { status = YGPU_ERR_TIMEOUT; goto out_; }
    }
    if (mixed) {
        // the FP32 copies of the operator coefficients and the Jacobi diagonal
        // were written by the phases that produce them; the tile-block
        // inverses of -p ilu are built from them here
        if (I.fminv && P.ssa_solver == YGPU_SSA_ENERGY && P.lin_precond == YGPU_PRE_ILU0) {
            const StencilOp<float, float> A32{&I, &G, true, I.fN, I.fNab, I.fdrag_x, I.fdrag_y, make_opk<float>(G)};
            block_setup<float, float>(I, G, T, A32, I.fminv);
            if (!team_barrier(T)) { status = YGPU_ERR_TIMEOUT; goto out_; }
        }
    }
    t4 = clk.lap();
out_:
    if (lead) {
        out->phase_ns[1] += t1;
        out->phase_ns[2] += t2;
        out->phase_ns[3] += t3;
        out->phase_ns[4] += t4;
        out->iter_now = iter;
        out->in_alt = in_alt ^ 1;
        out->bn2 = bn2;
        if (status != YGPU_OK) {
            out->status = status;
            out->done = 1;
            atomicAdd(done_count, 1);
        }
    }
}

__device__ __noinline__ void step_krylov(const Inst& I, const ygpu_dyn_par& P, Team& T, int* done_count) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    const Geo G = make_geo(I, P);
    InstOut* out = I.out;
    const bool lead = (T.cta == 0 && threadIdx.x == 0);
    PhaseClock clk;
    clk.start();
    const unsigned long long s0 = T.sync_ns;
    const double bn2 = out->bn2;
    int it = 0, outer = 0, st;
    double rr = 0.0;
    bool ok = true;
    if (bn2 == 0.0) {
        // homogeneous system: x = 0 (solver_linear.F90:162-174)
        for (int u = t_tid; u < G.nu; u += t_nthr) I.x[u] = 0.0;
        st = YGPU_OK;
    } else {
        st = linear_solve(I, P, G, T, sqrt(bn2), it, rr, outer, ok);
    }
    if (ok) ok = team_barrier(T);
    if (lead) {
        out->phase_ns[5] += clk.lap();
        out->phase_ns[9] += (double)(T.sync_ns - s0);
        out->lin_it = it;
        out->lin_st = st;
        out->lin_outer = outer;
        out->lin_rr = rr;
        if (!ok) {
            out->status = YGPU_ERR_TIMEOUT;
            out->done = 1;
            atomicAdd(done_count, 1);
        }
    }
}

// passes after the Picard loop (also for ssa_iter_max = 0)
__device__ __noinline__ bool final_passes(const Inst& I, const ygpu_dyn_par& P, const Geo& G, Team& T, bool diva,
                                          int in_alt, bool looped) {
    const int t_tid = T.tid, t_nthr = T.nthr;   // registers: the Team lives in the stack frame
    if (P.precision == YGPU_PREC_MIXED) {
        // the final FP32 viscosity goes to the caller's FP64 array first; the
        // passes below then read it there
        if (looped) {
            const size_t n3 = (size_t)G.n2 * G.nz;
            const float* vf = (const float*)I.visc_alt + (in_alt ? n3 : 0);
            for (size_t k = t_tid; k < n3; k += t_nthr) I.visc[k] = (double)vf[k];
            if (diva) {
                // the shear of the last iteration, kept in FP32 by the loop
                const float* sx = shear_f32(I, 0);
                const float* sy = shear_f32(I, 1);
                for (size_t k = t_tid; k < n3; k += t_nthr) {
                    I.duxdz[k] = (double)sx[k];
                    I.duydz[k] = (double)sy[k];
                }
            }
            if (!team_barrier(T)) return false;
        }
        in_alt = 0;
        looped = false;
    }
    double* vcur = in_alt ? I.visc_alt : I.visc;
    // viscosity of the last linear system (before the last update)
    const double* vlast = looped ? (in_alt ? I.visc : I.visc_alt) : vcur;
    double* sdudx = I.lk_x;
    double* sdudy = I.lk_y;
    double* sdvdx = I.lr_x;
    double* sdvdy = I.lr_y;
    double nlim = count_lim_part(I, P, G, T);
    if (diva) {
        phase_diva_final(I, G, T, vlast, vcur);
    } else {
        for (int c = t_tid; c < G.n2; c += t_nthr) {
            // calc_basal_stress, velocity_ssa.f90:588-617
            double tx = I.bm_x[c] * I.u_x[c], ty = I.bm_y[c] * I.u_y[c];
            I.taub_x[c] = (fabs(tx) < 1e-5) ? 0.0 : tx;
            I.taub_y[c] = (fabs(ty) < 1e-5) ? 0.0 : ty;
        }
    }
    if (!team_allreduce(T, &nlim, 1)) return false;
    if (!diva && P.visc_method == 0) {
        // diagnose the viscosity of the solution (not used prognostically)
        phase_strain(I, G, T, I.u_x, I.u_y, sdudx, sdudy, sdvdx, sdvdy);
        if (!team_barrier(T)) return false;
        ygpu_dyn_par P1 = P;
        P1.visc_method = 1;
        P1.precision = YGPU_PREC_FP64;     // the diagnostic pass reads FP64 powers
        phase_att_powers(I, P1, G, T);
        if (!team_barrier(T)) return false;
        phase_column<double, double>(I, P1, G, T, vcur, vcur, sdudx, sdudy, sdvdx, sdvdy, false, false, false, false, true);
        if (!team_barrier(T)) return false;
    }
    // the caller's visc_eff must hold the final viscosity
    if (in_alt) {
        for (size_t k = t_tid; k < (size_t)G.n2 * G.nz; k += t_nthr) I.visc[k] = I.visc_alt[k];
    }
    if (T.cta == 0 && threadIdx.x == 0) I.out->lim_n = (int)nlim;
    return team_barrier(T);
}

__device__ __noinline__ void step_post(const Inst& I, const ygpu_dyn_par& P, Team& T, int* done_count, bool final_only) {
    const bool diva = (I.kind == YGPU_KIND_DIVA);
    const Geo G = make_geo(I, P);
    InstOut* out = I.out;
    const bool lead = (T.cta == 0 && threadIdx.x == 0);
    PhaseClock clk;
    clk.start();
    int status = YGPU_OK;
    bool finish = final_only;
    double resid = out->resid;
    if (!final_only) {
        double red[4];
        phase_epilogue(I, P, G, T, diva, red);
        if (!team_allreduce(T, red, 4)) status = YGPU_ERR_TIMEOUT;
        resid = (red[2] > 0.0) ? sqrt(red[0]) / (sqrt(red[1]) + 1e-10) : 0.0;
        if (P.ssa_write_log && lead)
            printf("ssa: %s %4d %12.4g | lin %6d %d\n", (resid < P.ssa_iter_conv) ? "C" : "", out->iter_now, resid,
                   out->lin_it, out->lin_st);
        if (status == YGPU_OK && (red[3] > 0.0 || !isfinite(resid))) status = YGPU_ERR_NONFINITE;
        finish = (status != YGPU_OK) || resid < P.ssa_iter_conv || out->iter_now >= P.ssa_iter_max;
        // with a host hook between iterations the host decides (it may find the
        // hook's fields still changing); errors finish at once
        if (finish && status == YGPU_OK && out->defer) {
            if (lead) out->want_finish = 1;
            finish = false;
        }
    }
    const double t6 = clk.lap();
    // the last iteration's relative change (nothing on the device reads it)
    if (finish && out->iter_now > 0) phase_err(I, G, T);
    if (finish && status == YGPU_OK) {
        if (!final_passes(I, P, G, T, diva, out->in_alt, out->iter_now > 0)) status = YGPU_ERR_TIMEOUT;
    }
    const double t7 = clk.lap();
    if (lead) {
        if (!final_only) {
            out->lin_iter += out->lin_it;
            out->outer_iter += out->lin_outer;
            if (out->lin_st != YGPU_OK) out->lin_fail++;
            out->lin_status = out->lin_st;
            out->lin_resid = out->lin_rr;
            out->resid = resid;
        }
        out->phase_ns[6] += t6;
        out->phase_ns[7] += t7;
        if (finish) {
            out->status = (status != YGPU_OK) ? status : out->lin_status;
            out->converged = (status == YGPU_OK);
            out->done = 1;
            atomicAdd(done_count, 1);
        }
    }
}

// ---------------------------------------------------------------------------
// Step kernels: teams of CTAs, instances assigned round-robin in queue order
// ---------------------------------------------------------------------------

// Team layout of a launch: uniform teams of team_ctas CTAs taking instances
// round-robin, or (map != NULL) one team per instance with its own CTA count:
// map[cta] = instance of the CTA (-1: idle), map[grid + 2q] / [grid + 2q + 1] =
// first CTA and CTA count of instance q's team.
template <int STEP>
YG_DEV void run_step(const Inst* insts, int n_inst, const ygpu_dyn_par& P, TeamCtl* ctls, int team_ctas,
                     int* abort_all, int* done_count, const int* map) {
    __shared__ Inst sI;
    __shared__ int s_skip;
    Team T;
    int team, n_teams;
    if (map) {
        team = map[blockIdx.x];
        if (team < 0) return;
        const int* tm = map + gridDim.x + 2 * team;
        T.ncta = tm[1];
        T.cta = blockIdx.x - tm[0];
        n_teams = n_inst;          // the loop below visits instance `team` only
    } else {
        T.ncta = team_ctas;
        T.cta = blockIdx.x % team_ctas;
        team = blockIdx.x / team_ctas;
        n_teams = gridDim.x / team_ctas;
    }
    T.tid = T.cta * blockDim.x + threadIdx.x;
    T.nthr = T.ncta * blockDim.x;
    T.ctl = ctls + team;
    T.parity = 0;
    T.abort_all = abort_all;
    T.sync_ns = 0ull;
    T.gen = (threadIdx.x == 0) ? ld_acquire_u32(&T.ctl->base) : 0u;
    T.agen = ld_acquire_u32(&T.ctl->abase);
    T.spin_lim = team_spin_limit(T.ctl);
    T.cl = false;
    for (int q = team; q < n_inst; q += n_teams) {
        if (threadIdx.x == 0) {
            sI = insts[q];
            const int d = sI.out->done;
            s_skip = (STEP == YG_STEP_SETUP) ? 0 : (d || ld_acquire_s32(abort_all));
        }
        __syncthreads();
        if (!s_skip) {
            if (STEP == YG_STEP_SETUP) step_setup(sI, P, T, done_count);
            else if (STEP == YG_STEP_PRE) step_pre(sI, P, T, done_count);
            else if (STEP == YG_STEP_KRYLOV) step_krylov(sI, P, T, done_count);
            else step_post(sI, P, T, done_count, STEP == YG_STEP_FINAL);
            if (T.cta == 0 && threadIdx.x == 0) sI.out->phase_ns[8] += T.sync_ns;
            T.sync_ns = 0ull;
        }
        __syncthreads();
    }
    if (T.cta == 0 && threadIdx.x == 0) {
        T.ctl->base = T.gen;
        T.ctl->abase = T.agen;
    }
}

#define YG_KBLOCK 512
// the mixed-precision pre step (FP32 column pass, faces, system) runs 512-thread
// CTAs at 128 registers: twice the warps per SM of 256 threads at 255 registers
#define YG_PBLOCK 512

__global__ void __launch_bounds__(YG_BLOCK, 1) ygpu_k_setup(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                            TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_SETUP>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
__global__ void __launch_bounds__(YG_PBLOCK, 1) ygpu_k_pre(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                          TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_PRE>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
// the same pre step on 1024-thread CTAs (64 registers), for batches whose CTAs
// hold many cells (StepShape::wide_pre)
#define YG_PBLOCK_W 1024
__global__ void __launch_bounds__(YG_PBLOCK_W, 1) ygpu_k_pre_w(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                          TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_PRE>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
// FP64 solves: the FP64 column pass needs the full register file (256 threads)
__global__ void __launch_bounds__(YG_BLOCK, 1) ygpu_k_pre64(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                          TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_PRE>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
__global__ void __launch_bounds__(YG_KBLOCK, 1) ygpu_k_krylov(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                              TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_KRYLOV>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
// The Krylov step with every team one thread-block cluster (cluster size =
// team size, at most 16 CTAs): the team barrier is the hardware cluster barrier
// and the all-reduce reads the other CTAs' totals from their shared memory, with
// no global control block or polling. Cluster c takes instances c, c + n_clusters,
// ... The skip decision is the same in every CTA of a cluster: the instance's
// done flag (not written during this step) and the abort flag as CTA 0 of the
// cluster reads it once. Every barrier of a cluster team completes (its CTAs run
// the same control flow on identical all-reduced values), so no wait here needs
// a spin limit.
__global__ void __launch_bounds__(YG_KBLOCK, 1) ygpu_k_krylov_cl(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                                 TeamCtl* ctls, int tc, int* ab, int* dc,
                                                                 const int* map) {
    namespace cgx = cooperative_groups;
    cgx::cluster_group cl = cgx::this_cluster();
    __shared__ Inst sI;
    __shared__ int s_flags[2];     // [0] this CTA's abort read (rank 0's is used), [1] skip
    Team T;
    T.ncta = (int)cl.num_blocks();
    T.cta = (int)cl.block_rank();
    const int team = blockIdx.x / T.ncta, n_teams = gridDim.x / T.ncta;
    T.tid = T.cta * blockDim.x + threadIdx.x;
    T.nthr = T.ncta * blockDim.x;
    T.ctl = ctls;                  // not used by cluster teams
    T.parity = 0;
    T.abort_all = ab;
    T.sync_ns = 0ull;
    T.gen = 0u;
    T.agen = 0u;
    T.spin_lim = YG_SPIN_LIMIT;
    T.cl = true;
    if (threadIdx.x == 0) s_flags[0] = ld_acquire_s32(ab);
    cl.sync();
    const int aborted = *cl.map_shared_rank(&s_flags[0], 0);
    for (int q = team; q < n_inst; q += n_teams) {
        if (threadIdx.x == 0) {
            sI = insts[q];
            s_flags[1] = sI.out->done || aborted;
        }
        __syncthreads();
        if (!s_flags[1]) {
            step_krylov(sI, P, T, dc);
            if (T.cta == 0 && threadIdx.x == 0) sI.out->phase_ns[8] += T.sync_ns;
            T.sync_ns = 0ull;
        }
        // no CTA starts the next instance (or leaves) while another may still read
        // its shared memory
        cl.sync();
    }
    // every CTA has read CTA 0's abort flag before any of them leaves
    cl.sync();
}

// the post step (epilogue of a Picard iteration) runs 512-thread CTAs: twice the warps
// per SM of 256 threads, for a pass bound by load latency
#define YG_POBLOCK 512
__global__ void __launch_bounds__(YG_POBLOCK, 1) ygpu_k_post(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                           TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_POST>(insts, n_inst, P, ctls, tc, ab, dc, map);
}
__global__ void __launch_bounds__(YG_BLOCK, 1) ygpu_k_final(const Inst* insts, int n_inst, ygpu_dyn_par P,
                                                            TeamCtl* ctls, int tc, int* ab, int* dc, const int* map) {
    run_step<YG_STEP_FINAL>(insts, n_inst, P, ctls, tc, ab, dc, map);
}

// ---------------------------------------------------------------------------
// CSR seam: one team (the grid) solves A x = b with the LIS option semantics
// ---------------------------------------------------------------------------
struct CsrJob {
    int n, method, precond, maxiter, initx_zeros;
    double tol;
    const int *ptr, *idx;
    const double *val, *b;
    double *x, *dinv, *r, *rt, *p, *q, *v, *s, *t, *ph, *sh, *z;
    int* out_iters;
    int* out_status;
    double* out_relres;
};

__global__ void __launch_bounds__(YG_BLOCK) ygpu_csr_kernel(CsrJob J, TeamCtl* ctl, int* abort_all) {
    Team T;
    T.ncta = gridDim.x;
    T.cta = blockIdx.x;
    T.tid = blockIdx.x * blockDim.x + threadIdx.x;
    T.nthr = gridDim.x * blockDim.x;
    T.ctl = ctl;
    T.parity = 0;
    T.abort_all = abort_all;
    T.sync_ns = 0ull;
    T.gen = 0u;
    T.agen = 0u;
    T.spin_lim = YG_SPIN_LIMIT;
    T.cl = false;
    const bool lead = (blockIdx.x == 0 && threadIdx.x == 0);
    // Jacobi diagonal and ||b||
    double bn = 0.0;
    for (int r = T.tid; r < J.n; r += T.nthr) {
        double d = 0.0;
        for (int k = J.ptr[r]; k < J.ptr[r + 1]; k++)
            if (J.idx[k] == r) d += J.val[k];
        if (J.method == YGPU_LIN_MINRES) d = fabs(d);
        J.dinv[r] = (d != 0.0) ? 1.0 / d : 1.0;
        if (J.initx_zeros) J.x[r] = 0.0;
        bn += J.b[r] * J.b[r];
    }
    if (!team_allreduce(T, &bn, 1)) {
        if (lead) *J.out_status = YGPU_ERR_TIMEOUT;
        return;
    }
    int iters = 0, st;
    double rel = 0.0;
    bool ok = true;
    if (bn == 0.0) {
        for (int r = T.tid; r < J.n; r += T.nthr) J.x[r] = 0.0;
        st = YGPU_OK;
    } else {
        const CsrOp A{J.n, J.ptr, J.idx, J.val};
        const bool pre = (J.precond != YGPU_PRE_NONE);
        if (J.method == YGPU_LIN_BICGSTAB)
            st = krylov_bicgstab<double>(T, J.n, A, J.dinv, J.x, J.b, J.r, J.rt, J.p, J.v, J.s, J.t, J.ph, J.sh,
                                         J.maxiter, J.tol, sqrt(bn), pre, iters, rel, ok);
        else
            st = krylov_cg<double>(T, J.n, A, J.dinv, J.x, J.b, J.r, J.p, J.q, J.z, J.maxiter, J.tol, sqrt(bn), pre,
                                   iters, rel, ok);
        if (!ok) st = YGPU_ERR_TIMEOUT;
    }
    if (lead) {
        *J.out_iters = iters;
        *J.out_status = st;
        *J.out_relres = rel;
    }
}

int ygpu_launch_csr(cudaStream_t stream, int n, const int* ptr, const int* idx, const double* val, const double* b,
                    double* x, double* work, int method, int precond, int maxiter, double tol, int initx_zeros,
                    int* d_out_i, double* d_out_d, TeamCtl* d_ctl, int* d_abort, int n_ctas) {
    CsrJob J;
    J.n = n; J.method = method; J.precond = precond; J.maxiter = maxiter; J.initx_zeros = initx_zeros; J.tol = tol;
    J.ptr = ptr; J.idx = idx; J.val = val; J.b = b; J.x = x;
    double* w[12];
    for (int k = 0; k < 12; k++) w[k] = work + (size_t)k * n;
    J.dinv = w[0]; J.r = w[1]; J.rt = w[2]; J.p = w[3]; J.q = w[4]; J.v = w[5]; J.s = w[6]; J.t = w[7];
    J.ph = w[8]; J.sh = w[9]; J.z = w[10];
    J.out_iters = d_out_i;
    J.out_status = d_out_i + 1;
    J.out_relres = d_out_d;
    if (cudaMemsetAsync(d_abort, 0, sizeof(int), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    if (cudaMemsetAsync(d_ctl, 0, sizeof(TeamCtl), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    void* args[] = {(void*)&J, (void*)&d_ctl, (void*)&d_abort};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)ygpu_csr_kernel, dim3(n_ctas), dim3(YG_BLOCK), args, 0,
                                                stream);
    if (e != cudaSuccess) {
        ygpu_set_error("cooperative launch of the CSR solve failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

// ---------------------------------------------------------------------------
// Implicit upwind advection: calc_advec2D(solver = "impl-lis")
// (solver_advection.f90:20-145): the system of
// linear_solver_matrix_advection_csr_2D (:171-487), solved with BiCGSTAB and
// Jacobi to 1e-12 (the option string of :119), then the transport of the
// prescribed cells (calc_fixed_cell_transport, :489-546) and dvdt.
// ---------------------------------------------------------------------------
enum { ADV_PERIODIC = 0, ADV_ZERO = 1, ADV_INFINITE = 2, ADV_OUTFLOW = 3 };
#define YG_MASK_ICE_NONE 0
#define YG_MASK_ICE_FIXED 1

// define_advection_bcs (:548-622): kinds of the right, upper, left, lower borders
YG_DEV void adv_border_kinds(int code, int k[4]) {
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

struct AdvJob {
    int nx, ny, code;                  // YGPU_BND_* or YGPU_BND_MASK
    double dx, dy, dt;
    const double *var, *ux, *uy, *F, *Href;
    const int* mask;
    double* dvdt;
    double *c, *x, *b, *dinv, *r, *rt, *p, *v, *s, *t, *ph, *sh;   // c: 5 per row
    int* out_iters;
    int* out_status;
    double* out_relres;
};

// Face velocities of cell (i, j) after limit_border_inflow (:646-668): no flow
// from an "outflow" border cell into its inner neighbour
struct AdvFaces {
    double ux1, ux2, uy1, uy2;
};
YG_DEV double adv_ux(const AdvJob& J, const int* k, int i, int j) {
    double u = J.ux[i + J.nx * j];
    if (k[2] == ADV_OUTFLOW && i == 0 && u > 0.0) u = 0.0;
    if (k[0] == ADV_OUTFLOW && i == J.nx - 2 && u < 0.0) u = 0.0;
    return u;
}
YG_DEV double adv_uy(const AdvJob& J, const int* k, int i, int j) {
    double u = J.uy[i + J.nx * j];
    if (k[3] == ADV_OUTFLOW && j == 0 && u > 0.0) u = 0.0;
    if (k[1] == ADV_OUTFLOW && j == J.ny - 2 && u < 0.0) u = 0.0;
    return u;
}
// calc_upwind_faces (:670-755) for cell (i, j): the velocities of its four
// faces (1: left/bottom, 2: right/top) and the upstream values of H there
YG_DEV AdvFaces adv_faces(const AdvJob& J, const int* k, int i, int j, const double* H, double Hf[4]) {
    const int nx = J.nx, ny = J.ny;
    const int bc = (J.code == YGPU_BND_MASK) ? YGPU_BND_INFINITE : J.code;
    int im1, ip1, jm1, jp1;
    nbr_bc(i, j, nx, ny, bc, im1, ip1, jm1, jp1);
    AdvFaces f;
    f.ux1 = adv_ux(J, k, im1, j);
    f.ux2 = adv_ux(J, k, i, j);
    f.uy1 = adv_uy(J, k, i, jm1);
    f.uy2 = adv_uy(J, k, i, j);
    if (i == 0 && k[2] != ADV_PERIODIC) f.ux1 = 0.0;
    if (i == nx - 1 && k[0] != ADV_PERIODIC) f.ux2 = 0.0;
    if (j == 0 && k[3] != ADV_PERIODIC) f.uy1 = 0.0;
    if (j == ny - 1 && k[1] != ADV_PERIODIC) f.uy2 = 0.0;
    const int c = i + nx * j;
    Hf[0] = (f.ux1 >= 0.0) ? H[im1 + nx * j] : H[c];
    Hf[1] = (f.ux2 >= 0.0) ? H[c] : H[ip1 + nx * j];
    Hf[2] = (f.uy1 >= 0.0) ? H[i + nx * jm1] : H[c];
    Hf[3] = (f.uy2 >= 0.0) ? H[c] : H[i + nx * jp1];
    return f;
}

// The advection matrix: five coefficients per row in the slot order of the
// assembly, S (i,j-1), W (i-1,j), C, E (i+1,j), N (i,j+1), with columns wrapped
// periodically as there (border rows only use in-range columns)
struct Adv5Op {
    int nx, ny, n;
    const double* c;
    const int* acell = nullptr;        // every row
    YG_DEV int n2() const { return n; }
    YG_DEV double row(int r, const double* v) const {
        const int i = r % nx, j = r / nx;
        const int im1 = (i == 0) ? nx - 1 : i - 1, ip1 = (i == nx - 1) ? 0 : i + 1;
        const int jm1 = (j == 0) ? ny - 1 : j - 1, jp1 = (j == ny - 1) ? 0 : j + 1;
        const double* a = c + 5 * (size_t)r;
        double y = a[0] * v[i + nx * jm1];
        y = y + a[1] * v[im1 + nx * j];
        y = y + a[2] * v[r];
        y = y + a[3] * v[ip1 + nx * j];
        y = y + a[4] * v[i + nx * jp1];
        return y;
    }
    YG_DEV void operator()(Team& Tm, const double* v, double* y) const {
        for (int r = Tm.tid; r < n; r += Tm.nthr) y[r] = row(r, v);
    }
    YG_DEV void apply(Team& Tm, const double* v, double* y, const RowItems& R) const {
        int q = 0;
        for (int t = R.t0; t < R.t1; t += R.ts, q++) {
            const int k = R.row(t, q);
            y[k] = row(k, v);
        }
    }
};

__global__ void __launch_bounds__(YG_BLOCK) ygpu_adv_kernel(AdvJob J, TeamCtl* ctl, int* abort_all) {
    Team T;
    T.ncta = gridDim.x;
    T.cta = blockIdx.x;
    T.tid = blockIdx.x * blockDim.x + threadIdx.x;
    T.nthr = gridDim.x * blockDim.x;
    T.ctl = ctl;
    T.parity = 0;
    T.abort_all = abort_all;
    T.sync_ns = 0ull;
    T.gen = 0u;
    T.agen = 0u;
    T.spin_lim = YG_SPIN_LIMIT;
    T.cl = false;
    const bool lead = (blockIdx.x == 0 && threadIdx.x == 0);
    const int nx = J.nx, ny = J.ny, n = nx * ny;
    int k[4];
    adv_border_kinds(J.code, k);
    const bool row_bc[4] = {k[0] == ADV_ZERO || k[0] == ADV_INFINITE, k[1] == ADV_ZERO || k[1] == ADV_INFINITE,
                            k[2] == ADV_ZERO || k[2] == ADV_INFINITE, k[3] == ADV_ZERO || k[3] == ADV_INFINITE};
    const double dt_darea = J.dt / (J.dx * J.dy);
    const double WOVI = 1.0;
    // rows of linear_solver_matrix_advection_csr_2D (:258-481)
    double bn = 0.0;
    for (int r = T.tid; r < n; r += T.nthr) {
        const int i = r % nx, j = r / nx;
        double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
        double b, x0;
        const int m = J.mask[r];
        const bool use_border_bc = (m != YG_MASK_ICE_NONE);
        const double H = J.var[r];
        if (m == YG_MASK_ICE_FIXED) {
            a[2] = 1.0;
            b = J.Href[r];
            x0 = J.Href[r];
        } else if (use_border_bc && row_bc[0] && i == nx - 1) {          // right
            a[2] = 1.0;
            if (k[0] == ADV_INFINITE) { a[1] = -1.0; b = 0.0; x0 = H; } else { b = 0.0; x0 = 0.0; }
        } else if (use_border_bc && row_bc[1] && j == ny - 1) {          // top
            a[2] = 1.0;
            if (k[1] == ADV_INFINITE) { a[0] = -1.0; b = 0.0; x0 = H; } else { b = 0.0; x0 = 0.0; }
        } else if (use_border_bc && row_bc[2] && i == 0) {               // left
            a[2] = 1.0;
            if (k[2] == ADV_INFINITE) { a[3] = -1.0; b = 0.0; x0 = H; } else { b = 0.0; x0 = 0.0; }
        } else if (use_border_bc && row_bc[3] && j == 0) {               // bottom
            a[2] = 1.0;
            if (k[3] == ADV_INFINITE) { a[4] = -1.0; b = 0.0; x0 = H; } else { b = 0.0; x0 = 0.0; }
        } else {                                                          // inner point
            double Hf[4];
            const AdvFaces f = adv_faces(J, k, i, j, J.var, Hf);
            if (f.uy1 > 0.0) a[0] = -(dt_darea * f.uy1 * J.dx * WOVI);
            if (f.ux1 > 0.0) a[1] = -(dt_darea * f.ux1 * J.dy * WOVI);
            a[2] = 1.0;
            if (f.uy1 < 0.0) a[2] = a[2] - dt_darea * f.uy1 * J.dx * WOVI;
            if (f.ux1 < 0.0) a[2] = a[2] - dt_darea * f.ux1 * J.dy * WOVI;
            if (f.ux2 > 0.0) a[2] = a[2] + dt_darea * f.ux2 * J.dy * WOVI;
            if (f.uy2 > 0.0) a[2] = a[2] + dt_darea * f.uy2 * J.dx * WOVI;
            if (f.ux2 < 0.0) a[3] = dt_darea * f.ux2 * J.dy * WOVI;
            if (f.uy2 < 0.0) a[4] = dt_darea * f.uy2 * J.dx * WOVI;
            const double fx = f.ux2 * Hf[1] * J.dy - f.ux1 * Hf[0] * J.dy;
            const double fy = f.uy2 * Hf[3] * J.dx - f.uy1 * Hf[2] * J.dx;
            b = H + J.dt * J.F[r] - (1.0 - WOVI) * dt_darea * (fx + fy);
            x0 = H;
        }
        for (int q = 0; q < 5; q++) J.c[5 * (size_t)r + q] = a[q];
        J.b[r] = b;
        J.x[r] = x0;
        J.dinv[r] = (a[2] != 0.0) ? 1.0 / a[2] : 1.0;
        bn += b * b;
    }
    if (!team_allreduce(T, &bn, 1)) {
        if (lead) { *J.out_status = YGPU_ERR_TIMEOUT; *J.out_iters = 0; *J.out_relres = 0.0; }
        return;
    }
    int iters = 0, status = YGPU_OK;
    double relres = 0.0;
    bool ok = true;
    if (bn == 0.0) {
        // homogeneous system: x = 0 (solver_linear.F90:162-174)
        for (int r = T.tid; r < n; r += T.nthr) J.x[r] = 0.0;
    } else {
        const Adv5Op A{nx, ny, n, J.c};
        status = krylov_bicgstab<double>(T, n, A, J.dinv, J.x, J.b, J.r, J.rt, J.p, J.v, J.s, J.t, J.ph, J.sh, 1000,
                                         1e-12, sqrt(bn), true, iters, relres, ok);
        if (!ok) status = YGPU_ERR_TIMEOUT;
    }
    if (!team_barrier(T)) status = YGPU_ERR_TIMEOUT;
    // linear_solver_save_advection, calc_fixed_cell_transport on the solution, dvdt
    for (int r = T.tid; r < n; r += T.nthr) {
        double vn = J.x[r];
        if (J.mask[r] == YG_MASK_ICE_FIXED) {
            const int i = r % nx, j = r / nx;
            double Hf[4];
            const AdvFaces f = adv_faces(J, k, i, j, J.x, Hf);
            vn = J.var[r] + J.dt * J.F[r] -
                 dt_darea * ((f.ux2 * Hf[1] - f.ux1 * Hf[0]) * J.dy + (f.uy2 * Hf[3] - f.uy1 * Hf[2]) * J.dx);
        }
        J.dvdt[r] = (vn - J.var[r]) / J.dt;
    }
    if (lead) {
        *J.out_iters = iters;
        *J.out_status = status;
        *J.out_relres = relres;
    }
}

int ygpu_adv_max_ctas(int device) {
    int nsm = 0, bps = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ygpu_adv_kernel, YG_BLOCK, 0);
    return nsm * bps;
}

// work: 16 n doubles of device scratch
int ygpu_launch_advect(cudaStream_t stream, int nx, int ny, int code, double dx, double dy, double dt,
                       const double* var, const double* ux, const double* uy, const double* F, const double* Href,
                       const int* mask, double* dvdt, double* work, int* d_out_i, double* d_out_d, TeamCtl* d_ctl,
                       int* d_abort, int n_ctas) {
    AdvJob J;
    J.nx = nx; J.ny = ny; J.code = code; J.dx = dx; J.dy = dy; J.dt = dt;
    J.var = var; J.ux = ux; J.uy = uy; J.F = F; J.Href = Href; J.mask = mask; J.dvdt = dvdt;
    const size_t n = (size_t)nx * ny;
    J.c = work;
    double* w = work + 5 * n;
    double** slots[11] = {&J.x, &J.b, &J.dinv, &J.r, &J.rt, &J.p, &J.v, &J.s, &J.t, &J.ph, &J.sh};
    for (int q = 0; q < 11; q++) *slots[q] = w + (size_t)q * n;
    J.out_iters = d_out_i;
    J.out_status = d_out_i + 1;
    J.out_relres = d_out_d;
    if (cudaMemsetAsync(d_abort, 0, sizeof(int), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    if (cudaMemsetAsync(d_ctl, 0, sizeof(TeamCtl), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    void* args[] = {(void*)&J, (void*)&d_ctl, (void*)&d_abort};
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)ygpu_adv_kernel, dim3(n_ctas), dim3(YG_BLOCK), args, 0,
                                                stream);
    if (e != cudaSuccess) {
        ygpu_set_error("cooperative launch of the advection solve failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    ygpu_count_launches(1);
    return YGPU_OK;
}

int ygpu_csr_max_ctas(int device) {
    int nsm = 0, bps = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ygpu_csr_kernel, YG_BLOCK, 0);
    return nsm * bps;
}

// ---------------------------------------------------------------------------
// Host side: launch
// ---------------------------------------------------------------------------
static bool g_gqw_set[64] = {false};

// dynamic shared memory of the FP32 cell CG's record slots
static size_t krec_bytes(int slots) { return (size_t)slots * 4 * sizeof(float4) * YG_KBLOCK; }
// the Krylov kernel's dynamic shared memory limit, once per device (occupancy
// queries with the record slots need it set)
static bool set_smem_limits(int device) {
    static bool done[64] = {false};
    const int d = (device >= 0 && device < 64) ? device : 0;
    if (done[d]) return true;
    if (cudaFuncSetAttribute((const void*)ygpu_k_krylov, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)krec_bytes(YG_KREC_MAX)) != cudaSuccess) {
        ygpu_set_error("step kernels: dynamic shared memory limits refused");
        return false;
    }
    done[d] = true;
    return true;
}

static int max_ctas_of(const void* kern, int block, size_t smem = 0) {
    int dev = 0, nsm = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, block, smem);
    return nsm * bps;
}

static int coop(const void* kern, int grid, int block, cudaStream_t s, const Inst* insts, int n_inst,
                const ygpu_dyn_par& P, TeamCtl* ctls, int tc, int* ab, int* dc, const int* map, size_t smem = 0) {
    void* args[] = {(void*)&insts, (void*)&n_inst, (void*)&P, (void*)&ctls, (void*)&tc, (void*)&ab, (void*)&dc,
                    (void*)&map};
    cudaError_t e = cudaLaunchCooperativeKernel(kern, dim3(grid), dim3(block), args, smem, s);
    if (e != cudaSuccess) {
        ygpu_set_error("cooperative launch of a solver step failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    return YGPU_OK;
}

int ygpu_init_constants(int device) {
    if (device < 0 || device >= 64) return YGPU_OK;
    if (g_gqw_set[device]) return YGPU_OK;
    if (!set_smem_limits(device)) return YGPU_ERR_CUDA;
    double w[4][4];
    const int sx[4] = {-1, 1, 1, -1}, sy[4] = {-1, -1, 1, 1};
    const double g = 1.0 / sqrt(3.0);
    for (int q = 0; q < 4; q++)
        for (int c = 0; c < 4; c++) {
            volatile double ax = 1.0 + (double)(sx[q] * sx[c]) * g;
            volatile double ay = 1.0 + (double)(sy[q] * sy[c]) * g;
            volatile double pr = ax * ay;
            w[q][c] = pr * 0.25;
        }
    float wf[4][4];
    for (int q = 0; q < 4; q++)
        for (int c = 0; c < 4; c++) wf[q][c] = (float)w[q][c];
    if (cudaMemcpyToSymbol(c_gqw, w, sizeof(w)) != cudaSuccess) return YGPU_ERR_CUDA;
    if (cudaMemcpyToSymbol(c_gqwf, wf, sizeof(wf)) != cudaSuccess) return YGPU_ERR_CUDA;
    g_gqw_set[device] = true;
    return YGPU_OK;
}

int ygpu_step_shape_mapped(int device, int grid, const int* d_map, StepShape* sh) {
    // one team per instance with its own CTA count; the Krylov kernel uses the
    // same map when it has as many resident CTAs, else (kgrid = 0) the caller
    // must use a uniform shape
    static int kmax_dev[64];
    const int dslot = (device >= 0 && device < 64) ? device : 0;
    if (kmax_dev[dslot] == 0 && set_smem_limits(device))
        kmax_dev[dslot] = max_ctas_of((const void*)ygpu_k_krylov, YG_KBLOCK, krec_bytes(YG_KREC_MAX));
    if (kmax_dev[dslot] < grid) return YGPU_ERR_BAD_ARG;
    sh->grid = grid;
    sh->team_ctas = 1;
    sh->kgrid = grid;
    sh->ktc = 1;
    sh->map = d_map;
    sh->kmap = d_map;
    return YGPU_OK;
}

void ygpu_step_shape_wide(StepShape* sh, size_t total_unknowns) {
    sh->wide_pre = (sh->grid > 0 && total_unknowns / 2 > (size_t)sh->grid * 2 * YG_PBLOCK) ? 1 : 0;
    // shared-memory record slots of the FP32 cell CG: the cells per thread of the
    // Krylov step, rounded up, at most YG_KREC_MAX
    size_t per = 0;
    if (sh->kgrid > 0) per = (total_unknowns / 2 + (size_t)sh->kgrid * YG_KBLOCK - 1) / ((size_t)sh->kgrid * YG_KBLOCK);
    sh->kslots = (int)(per < YG_KREC_MAX ? per : YG_KREC_MAX);
}

int ygpu_step_shape(int device, int n_teams, int team_ctas, StepShape* sh) {
    sh->map = nullptr;
    sh->kmap = nullptr;
    // Krylov launch shape: the lean kernel; teams of as many CTAs as the heavy
    // teams (each CTA twice the threads), fewer teams if fewer CTAs are resident
    static int kmax_dev[64];
    const int dslot = (device >= 0 && device < 64) ? device : 0;
    if (kmax_dev[dslot] == 0 && set_smem_limits(device))
        kmax_dev[dslot] = max_ctas_of((const void*)ygpu_k_krylov, YG_KBLOCK, krec_bytes(YG_KREC_MAX));
    const int kmax = kmax_dev[dslot];
    if (kmax < 1) {
        ygpu_set_error("Krylov kernel cannot be resident on device %d", device);
        return YGPU_ERR_CUDA;
    }
    int ktc = team_ctas;
    if (ktc < 1) ktc = 1;
    if (ktc > kmax) ktc = kmax;
    int knt = kmax / ktc;
    if (knt > n_teams) knt = n_teams;
    sh->team_ctas = team_ctas;
    sh->grid = n_teams * team_ctas;
    sh->ktc = ktc;
    sh->kgrid = knt * ktc;
    return YGPU_OK;
}

// ---------------------------------------------------------------------------
// Launch accounting: a count of every kernel this library launches, and (when
// switched on) CUDA-event timing of each step launch on its own stream.
// ---------------------------------------------------------------------------
namespace {
std::atomic<unsigned long long> g_launches{0};
struct StepTimer {
    std::mutex mu;
    bool on = false;
    struct Rec { cudaEvent_t a, b; int kind; };
    std::vector<Rec> pending;
    std::vector<cudaEvent_t> spare;
    double ms[5] = {0, 0, 0, 0, 0};
    long long n[5] = {0, 0, 0, 0, 0};
    cudaEvent_t get() {
        if (!spare.empty()) {
            cudaEvent_t e = spare.back();
            spare.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }
} g_timer;
}  // namespace

void ygpu_count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

extern "C" unsigned long long ygpu_kernel_launches(void) { return g_launches.load(); }

extern "C" void ygpu_step_timing(int on) {
    std::lock_guard<std::mutex> lk(g_timer.mu);
    g_timer.on = (on != 0);
    if (on) {
        for (int k = 0; k < 5; k++) { g_timer.ms[k] = 0.0; g_timer.n[k] = 0; }
    }
}

// Folds the timed launches whose streams have finished into the totals.
void ygpu_step_timing_flush() {
    std::lock_guard<std::mutex> lk(g_timer.mu);
    std::vector<StepTimer::Rec> keep;
    for (auto& r : g_timer.pending) {
        if (cudaEventQuery(r.b) != cudaSuccess) {
            cudaGetLastError();
            keep.push_back(r);
            continue;
        }
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
            g_timer.ms[r.kind] += ms;
            g_timer.n[r.kind] += 1;
        }
        cudaGetLastError();
        g_timer.spare.push_back(r.a);
        g_timer.spare.push_back(r.b);
    }
    g_timer.pending.swap(keep);
}

void ygpu_step_timing_add(int kind, double ms) {
    std::lock_guard<std::mutex> lk(g_timer.mu);
    if (!g_timer.on || kind < 0 || kind >= 5) return;
    g_timer.ms[kind] += ms;
    g_timer.n[kind] += 1;
}

extern "C" void ygpu_step_timing_get(double ms[5], long long count[5]) {
    ygpu_step_timing_flush();
    std::lock_guard<std::mutex> lk(g_timer.mu);
    for (int k = 0; k < 5; k++) {
        if (ms) ms[k] = g_timer.ms[k];
        if (count) count[k] = g_timer.n[k];
    }
}

static int launch_step_raw(int step, cudaStream_t s, const StepShape& sh, const Inst* d_insts, int n_inst,
                           const ygpu_dyn_par& P, TeamCtl* ctls, int* d_done, int* d_abort);

int ygpu_launch_step(int step, cudaStream_t s, const StepShape& sh, const Inst* d_insts, int n_inst,
                     const ygpu_dyn_par& P, TeamCtl* ctls, int* d_done, int* d_abort) {
    cudaEvent_t a = nullptr, b = nullptr;
    bool timed = false;
    if (step >= 0 && step < 5) {
        std::lock_guard<std::mutex> lk(g_timer.mu);
        if (g_timer.on) {
            a = g_timer.get();
            b = g_timer.get();
            timed = (a && b);
        }
    }
    if (timed) cudaEventRecord(a, s);
    const int st = launch_step_raw(step, s, sh, d_insts, n_inst, P, ctls, d_done, d_abort);
    if (st == YGPU_OK) ygpu_count_launches(1);
    if (timed) {
        cudaEventRecord(b, s);
        std::lock_guard<std::mutex> lk(g_timer.mu);
        g_timer.pending.push_back({a, b, step});
    }
    return st;
}

// The Krylov step on cluster teams: an ordinary launch with a cluster dimension
// (the CTAs of a cluster are co-scheduled by the hardware; clusters do not wait
// on one another, so no cooperative launch is needed)
static int launch_cluster_krylov(cudaStream_t s, const StepShape& sh, const Inst* d_insts, int n_inst,
                                 const ygpu_dyn_par& P, TeamCtl* ctls, int* d_done, int* d_abort) {
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = (unsigned)sh.kcl;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.gridDim = dim3((unsigned)sh.kgrid);
    cfg.blockDim = dim3(YG_KBLOCK);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const int tc = sh.kcl;
    const int* map = nullptr;
    cudaError_t e = cudaLaunchKernelEx(&cfg, ygpu_k_krylov_cl, d_insts, n_inst, P, ctls, tc, d_abort, d_done, map);
    if (e != cudaSuccess) {
        ygpu_set_error("cluster launch of the Krylov step failed: %s", cudaGetErrorString(e));
        return YGPU_ERR_CUDA;
    }
    return YGPU_OK;
}

int ygpu_krylov_cluster_plan(int device, int n_inst, size_t max_nu, int req, int* n_clusters) {
    *n_clusters = 0;
    if (req < 2 || n_inst < 1 || device < 0 || device >= 64) return 0;
    static std::mutex mu;
    static int maxc[64][17];       // resident clusters per size (-1: not resident / not queried)
    static bool init[64];
    {
        std::lock_guard<std::mutex> lk(mu);
        if (!init[device]) {
            cudaFuncSetAttribute((const void*)ygpu_k_krylov_cl, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
            for (int cs = 1; cs <= 16; cs++) {
                cudaLaunchConfig_t cfg = {};
                cudaLaunchAttribute at[1];
                at[0].id = cudaLaunchAttributeClusterDimension;
                at[0].val.clusterDim.x = (unsigned)cs;
                at[0].val.clusterDim.y = 1;
                at[0].val.clusterDim.z = 1;
                cfg.gridDim = dim3((unsigned)cs);
                cfg.blockDim = dim3(YG_KBLOCK);
                cfg.attrs = at;
                cfg.numAttrs = 1;
                int n = 0;
                if (cudaOccupancyMaxActiveClusters(&n, (const void*)ygpu_k_krylov_cl, &cfg) != cudaSuccess) n = -1;
                maxc[device][cs] = n;
            }
            cudaGetLastError();
            init[device] = true;
        }
    }
    (void)max_nu;
    const int cs = req > 16 ? 16 : req;
    const int m = maxc[device][cs];
    if (m < 1) return 0;
    *n_clusters = (m < n_inst) ? m : n_inst;
    return cs;
}

static int launch_step_raw(int step, cudaStream_t s, const StepShape& sh, const Inst* d_insts, int n_inst,
                           const ygpu_dyn_par& P, TeamCtl* ctls, int* d_done, int* d_abort) {
    switch (step) {
        case YG_STEP_SETUP:
            return coop((const void*)ygpu_k_setup, sh.grid, YG_BLOCK, s, d_insts, n_inst, P, ctls, sh.team_ctas, d_abort, d_done, sh.map);
        case YG_STEP_PRE:
            if (P.precision == YGPU_PREC_MIXED && sh.wide_pre)
                return coop((const void*)ygpu_k_pre_w, sh.grid, YG_PBLOCK_W, s, d_insts, n_inst, P, ctls, sh.team_ctas,
                            d_abort, d_done, sh.map);
            if (P.precision == YGPU_PREC_MIXED)
                return coop((const void*)ygpu_k_pre, sh.grid, YG_PBLOCK, s, d_insts, n_inst, P, ctls, sh.team_ctas,
                            d_abort, d_done, sh.map);
            return coop((const void*)ygpu_k_pre64, sh.grid, YG_BLOCK, s, d_insts, n_inst, P, ctls, sh.team_ctas,
                        d_abort, d_done, sh.map);
        case YG_STEP_KRYLOV:
            if (sh.kcl > 0) return launch_cluster_krylov(s, sh, d_insts, n_inst, P, ctls, d_done, d_abort);
            return coop((const void*)ygpu_k_krylov, sh.kgrid, YG_KBLOCK, s, d_insts, n_inst, P, ctls, sh.ktc, d_abort, d_done,
                        sh.kmap, P.precision == YGPU_PREC_MIXED ? krec_bytes(sh.kslots) : 0);
        case YG_STEP_POST:
            return coop((const void*)ygpu_k_post, sh.grid, YG_POBLOCK, s, d_insts, n_inst, P, ctls, sh.team_ctas, d_abort, d_done, sh.map);
        case YG_STEP_FINAL:
            return coop((const void*)ygpu_k_final, sh.grid, YG_BLOCK, s, d_insts, n_inst, P, ctls, sh.team_ctas, d_abort, d_done, sh.map);
        default:
            ygpu_set_error("bad solver step %d", step);
            return YGPU_ERR_BAD_ARG;
    }
}

bool ygpu_step_timing_on() {
    std::lock_guard<std::mutex> lk(g_timer.mu);
    return g_timer.on;
}

void ygpu_graph_cache_clear(GraphCache* gc) {
    if (!gc) return;
    if (gc->exec) cudaGraphExecDestroy(gc->exec);
    for (auto& e : gc->ev) {
        cudaEventDestroy(e.a);
        cudaEventDestroy(e.b);
    }
    gc->ev.clear();
    gc->exec = nullptr;
    gc->valid = false;
}

// Captures `iters` Picard iterations (pre / Krylov / post launches) and the
// read-back of the finished count and abort flag into pinned host memory as
// one CUDA graph. Returns false (nothing captured, stream usable) on failure.
// With step timing on, every launch is bracketed by event-record nodes whose
// times are read after each replay.
static bool capture_chunk(cudaStream_t stream, const StepShape& sh, const Inst* d_insts, int n_inst,
                          const ygpu_dyn_par& P, TeamCtl* d_ctls, int* d_done, int* d_abort, int iters,
                          int* h_flags, GraphCache* gc, bool timed) {
    if (timed) {
        for (int k = 0; k < 3 * iters; k++) {
            GraphEvents e{nullptr, nullptr, YG_STEP_PRE + k % 3};
            if (cudaEventCreate(&e.a) != cudaSuccess || cudaEventCreate(&e.b) != cudaSuccess) {
                cudaGetLastError();
                if (e.a) cudaEventDestroy(e.a);
                if (e.b) cudaEventDestroy(e.b);
                return false;
            }
            gc->ev.push_back(e);
        }
    }
    cudaGraphExec_t* exec = &gc->exec;
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    bool ok = true;
    int k = 0;
    for (int it = 0; it < iters && ok; it++)
        for (int step : {YG_STEP_PRE, YG_STEP_KRYLOV, YG_STEP_POST}) {
            // external records: real event-record nodes of the graph (a plain record
            // inside a capture only orders the capture)
            if (ok && timed) ok = cudaEventRecordWithFlags(gc->ev[k].a, stream, cudaEventRecordExternal) == cudaSuccess;
            if (ok) ok = (launch_step_raw(step, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort) == YGPU_OK);
            if (ok && timed) ok = cudaEventRecordWithFlags(gc->ev[k].b, stream, cudaEventRecordExternal) == cudaSuccess;
            k++;
        }
    if (ok) ok = cudaMemcpyAsync(h_flags, d_done, sizeof(int), cudaMemcpyDeviceToHost, stream) == cudaSuccess;
    if (ok) ok = cudaMemcpyAsync(h_flags + 1, d_abort, sizeof(int), cudaMemcpyDeviceToHost, stream) == cudaSuccess;
    cudaGraph_t g = nullptr;
    const bool ended = cudaStreamEndCapture(stream, &g) == cudaSuccess;
    ok = ok && ended && g;
    if (ok) ok = cudaGraphInstantiate(exec, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return ok;
}

int ygpu_launch_solver(int device, cudaStream_t stream, const Inst* d_insts, int n_inst, const ygpu_dyn_par& P,
                       TeamCtl* d_ctls, int n_teams, int team_ctas, int* d_done, int* d_abort, const int* d_map,
                       int map_grid, GraphCache* gc, int* h_flags, int check_every, const NeffRun* hook,
                       int spin_log2, int cluster_req, size_t max_nu) {
    // d_done: count of finished instances; d_abort: launch-wide abort flag.
    // With a team map (one team per instance) n_teams is the number of control
    // blocks to clear (n_inst) and map_grid the CTAs of the plan.
    YgRange range("ygpu solve");
    int st;
    if ((st = ygpu_init_constants(device))) return st;
    if (cudaMemsetAsync(d_done, 0, sizeof(int), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    if (cudaMemsetAsync(d_abort, 0, sizeof(int), stream) != cudaSuccess) return YGPU_ERR_CUDA;
    if (cudaMemsetAsync(d_ctls, 0, sizeof(TeamCtl) * (size_t)n_teams, stream) != cudaSuccess) return YGPU_ERR_CUDA;
    // a lower spin budget for the team waits (tests of the timeout path)
    if (spin_log2 > 0 && cudaMemset2DAsync(&d_ctls[0].spin_log2, sizeof(TeamCtl), spin_log2, 1, (size_t)n_teams,
                                           stream) != cudaSuccess)
        return YGPU_ERR_CUDA;
    StepShape sh;
    if (d_map) st = ygpu_step_shape_mapped(device, map_grid, d_map, &sh);
    else st = ygpu_step_shape(device, n_teams, team_ctas, &sh);
    if (st) return st;
    ygpu_step_shape_wide(&sh, (size_t)n_inst * max_nu);
    // Krylov teams as thread-block clusters when every instance gets one resident cluster
    if (max_nu > 0) {
        int ncl = 0;
        const int cs = ygpu_krylov_cluster_plan(device, n_inst, max_nu, cluster_req, &ncl);
        if (cs > 0 && ncl > 0) {
            sh.kcl = cs;
            sh.kgrid = cs * ncl;
            sh.ktc = cs;
            sh.kmap = nullptr;
        }
    }
    if ((st = ygpu_launch_step(YG_STEP_SETUP, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort))) return st;
    // Picard iterations: one pre / Krylov / post launch each; the host reads the
    // count of finished instances every `check` iterations. With a graph cache
    // and pinned flags, each chunk of `check` iterations is one CUDA graph
    // (captured once per launch shape and parameters, then replayed).
    const int check = check_every > 0 ? check_every : 4;
    const bool use_graph = gc && h_flags && P.ssa_iter_max >= check && !hook;
    const bool timed = ygpu_step_timing_on();
    if (use_graph) {
        GraphKey key;
        memset(&key, 0, sizeof(key));
        key.insts = d_insts; key.n_inst = n_inst; key.sh = sh; key.ctls = d_ctls;
        memcpy(&key.P, &P, sizeof(P));   // bytes, padding included, for the memcmp below
        key.done = d_done; key.abort_ = d_abort; key.check = check; key.h_flags = h_flags;
        key.timed = timed;
        if (!gc->valid || memcmp(&gc->key, &key, sizeof(key)) != 0) {
            ygpu_graph_cache_clear(gc);
            if (capture_chunk(stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort, check, h_flags, gc, timed)) {
                memcpy(&gc->key, &key, sizeof(key));
                gc->valid = true;
            } else {
                ygpu_graph_cache_clear(gc);
            }
        }
    }
    int it = 0;
    if (hook) {
        // one iteration at a time, the host hook between iterations
        const size_t n2 = (size_t)hook->nx * hook->ny;
        for (; it < P.ssa_iter_max; it++) {
            for (int step : {YG_STEP_PRE, YG_STEP_KRYLOV, YG_STEP_POST})
                if ((st = ygpu_launch_step(step, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort))) return st;
            InstOut o;
            int ab = 0;
            if (cudaMemcpyAsync(&o, hook->d_out, sizeof(InstOut), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaMemcpyAsync(&ab, d_abort, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaMemcpyAsync(hook->h_uxb, hook->d_uxb, n2 * 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaMemcpyAsync(hook->h_uyb, hook->d_uyb, n2 * 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaMemcpyAsync(hook->h_cbed, hook->d_cbed, n2 * 8, cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaStreamSynchronize(stream) != cudaSuccess) {
                ygpu_set_error("solver step failed: %s", cudaGetErrorString(cudaGetLastError()));
                return YGPU_ERR_CUDA;
            }
            if (ab || o.done) break;
            // the hook, and the relative L1 change of c_bed (velocity_diva.f90:396-399)
            memcpy(hook->h_prev, hook->h_cbed, n2 * 8);
            hook->fn(hook->user, hook->h_cbed, hook->h_uxb, hook->h_uyb, hook->nx, hook->ny);
            double dsum = 0.0, csum = 0.0;
            for (size_t c = 0; c < n2; c++) {
                dsum += fabs(hook->h_cbed[c] - hook->h_prev[c]);
                csum += fabs(hook->h_cbed[c]);
            }
            const bool cb_converged = !(dsum > P.ssa_iter_conv * (csum > 1e-15 ? csum : 1e-15));
            if (cudaMemcpyAsync(hook->d_cbed, hook->h_cbed, n2 * 8, cudaMemcpyHostToDevice, stream) != cudaSuccess) {
                ygpu_set_error("c_bed upload failed: %s", cudaGetErrorString(cudaGetLastError()));
                return YGPU_ERR_CUDA;
            }
            if (o.want_finish && (cb_converged || o.iter_now >= P.ssa_iter_max)) break;   // final passes below
            if (o.want_finish) {
                const int zero = 0;
                if (cudaMemcpyAsync(&hook->d_out->want_finish, &zero, sizeof(int), cudaMemcpyHostToDevice, stream) !=
                        cudaSuccess ||
                    cudaStreamSynchronize(stream) != cudaSuccess) {
                    ygpu_set_error("solver state update failed: %s", cudaGetErrorString(cudaGetLastError()));
                    return YGPU_ERR_CUDA;
                }
            }
        }
        return ygpu_launch_step(YG_STEP_FINAL, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort);
    }
    if (use_graph && gc->valid) {
        // whole chunks as graph replays
        while (it + check <= P.ssa_iter_max) {
            YgRange chunk("ygpu picard chunk");
            if (cudaGraphLaunch(gc->exec, stream) != cudaSuccess || cudaStreamSynchronize(stream) != cudaSuccess) {
                ygpu_set_error("solver graph failed: %s", cudaGetErrorString(cudaGetLastError()));
                return YGPU_ERR_CUDA;
            }
            ygpu_count_launches(3ull * check);
            if (timed)
                for (const GraphEvents& e : gc->ev) {
                    float ms = 0.f;
                    if (cudaEventElapsedTime(&ms, e.a, e.b) == cudaSuccess) ygpu_step_timing_add(e.kind, ms);
                    cudaGetLastError();
                }
            it += check;
            if (h_flags[0] >= n_inst || h_flags[1]) {
                it = P.ssa_iter_max;
                break;
            }
        }
    }
    for (; it < P.ssa_iter_max; it++) {
        for (int step : {YG_STEP_PRE, YG_STEP_KRYLOV, YG_STEP_POST})
            if ((st = ygpu_launch_step(step, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort))) return st;
        if ((it + 1) % check == 0 || it + 1 == P.ssa_iter_max) {
            int h[2] = {0, 0};
            if (cudaMemcpyAsync(&h[0], d_done, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaMemcpyAsync(&h[1], d_abort, sizeof(int), cudaMemcpyDeviceToHost, stream) != cudaSuccess ||
                cudaStreamSynchronize(stream) != cudaSuccess) {
                ygpu_set_error("solver step failed: %s", cudaGetErrorString(cudaGetLastError()));
                return YGPU_ERR_CUDA;
            }
            if (h[0] >= n_inst || h[1]) break;
        }
    }
    // instances not finished by the loop (ssa_iter_max = 0) get their final passes
    return ygpu_launch_step(YG_STEP_FINAL, stream, sh, d_insts, n_inst, P, d_ctls, d_done, d_abort);
}

// Largest per-thread local memory (stack) of the step kernels, in bytes.
size_t ygpu_solver_stack_bytes() {
    const void* k[] = {(const void*)ygpu_k_setup, (const void*)ygpu_k_pre, (const void*)ygpu_k_pre_w,
                       (const void*)ygpu_k_pre64,
                       (const void*)ygpu_k_krylov, (const void*)ygpu_k_post, (const void*)ygpu_k_final};
    size_t m = 0;
    for (const void* f : k) {
        cudaFuncAttributes a;
        if (cudaFuncGetAttributes(&a, f) == cudaSuccess && a.localSizeBytes > m) m = a.localSizeBytes;
    }
    cudaGetLastError();
    return m;
}

int ygpu_solver_max_ctas(int device) {
    int nsm = 0, bps = 0, b2 = 0, b3 = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ygpu_k_pre, YG_PBLOCK, 0);
    int bw = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bw, ygpu_k_pre_w, YG_PBLOCK_W, 0);
    if (bw < bps) bps = bw;
    int b4 = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b4, ygpu_k_pre64, YG_BLOCK, 0);
    if (b4 < bps) bps = b4;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b2, ygpu_k_post, YG_POBLOCK, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b3, ygpu_k_setup, YG_BLOCK, 0);
    if (b2 < bps) bps = b2;
    if (b3 < bps) bps = b3;
    return nsm * bps;
}

int ygpu_sm_count(int device) {
    int nsm = 0;
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device);
    return nsm;
}

size_t ygpu_teamctl_bytes() { return sizeof(TeamCtl); }
size_t ygpu_inst_bytes() { return sizeof(Inst); }
