// ygpu_common.cuh -- device helpers shared by the sm_103a kernels:
// C-grid neighbour indexing with Yelmo's boundary codes, the instance
// descriptor the persistent solver works on, and the team barrier with a
// fused, deterministic all-reduce.
#pragma once

#include <cooperative_groups.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/yelmo_gpu.h"

#define YG_DEV __device__ __forceinline__

// ---------------------------------------------------------------------------
// Grid indexing (0-based, column-major: c = i + nx*j; 3D: c + n2*k)
// ---------------------------------------------------------------------------

// get_neighbor_indices_bc_codes, yelmo_tools.f90:118-201
YG_DEV void nbr_bc(int i, int j, int nx, int ny, int bc, int& im1, int& ip1, int& jm1, int& jp1) {
    const bool wx = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_X);
    const bool wy = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_Y || bc == YGPU_BND_MISMIP3D ||
                     bc == YGPU_BND_TROUGH);
    if (wx) {
        im1 = (i == 0) ? nx - 1 : i - 1;
        ip1 = (i == nx - 1) ? 0 : i + 1;
    } else {
        im1 = (i > 0) ? i - 1 : 0;
        ip1 = (i < nx - 1) ? i + 1 : nx - 1;
    }
    if (wy) {
        jm1 = (j == 0) ? ny - 1 : j - 1;
        jp1 = (j == ny - 1) ? 0 : j + 1;
    } else {
        jm1 = (j > 0) ? j - 1 : 0;
        jp1 = (j < ny - 1) ? j + 1 : ny - 1;
    }
}

YG_DEV void periodic_dirs(int bc, bool& px, bool& py) {
    px = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_X);
    py = (bc == YGPU_BND_PERIODIC || bc == YGPU_BND_PERIODIC_Y || bc == YGPU_BND_MISMIP3D ||
          bc == YGPU_BND_TROUGH);
}

// Border kinds of the assemblers (solver_ssa_ac.f90:149-210), index 0..3 =
// bcs(1..4) = right, upper, left, lower. Returns bits: periodic (1<<k), free (1<<(4+k)).
YG_DEV unsigned border_bits(int bc) {
    // 0 no-slip, 1 free-slip, 2 periodic
    int t0, t1, t2, t3;
    switch (bc) {
        case YGPU_BND_MISMIP3D:
        case YGPU_BND_TROUGH: t0 = 1; t1 = 2; t2 = 0; t3 = 2; break;
        case YGPU_BND_PERIODIC: t0 = t1 = t2 = t3 = 2; break;
        case YGPU_BND_PERIODIC_X: t0 = 2; t1 = 1; t2 = 2; t3 = 1; break;
        case YGPU_BND_PERIODIC_Y: t0 = 1; t1 = 2; t2 = 1; t3 = 2; break;
        case YGPU_BND_INFINITE: t0 = t1 = t2 = t3 = 1; break;
        default: t0 = t1 = t2 = t3 = 0; break;
    }
    unsigned b = 0;
    int t[4] = {t0, t1, t2, t3};
#pragma unroll
    for (int k = 0; k < 4; k++) {
        if (t[k] == 2) b |= 1u << k;
        if (t[k] == 1) b |= 1u << (4 + k);
    }
    return b;
}
YG_DEV bool bper(unsigned b, int k) { return (b >> k) & 1u; }
YG_DEV bool bfree(unsigned b, int k) { return (b >> (4 + k)) & 1u; }

// calc_staggered_margin, velocity_diva.f90:1052-1082
template <typename T>
YG_DEV T stag_margin(T v0, T v1, double f0, double f1) {
    if (f0 == 1.0 && f1 < 1.0) return v0;
    if (f0 < 1.0 && f1 == 1.0) return v1;
    return T(0.5) * (v0 + v1);
}

// ---------------------------------------------------------------------------
// Unknown numbering inside the GPU solver: two planes, ux then uy
//   u = c (ux at cell c) or n2 + c (uy at cell c)
// ---------------------------------------------------------------------------
enum { DOF_FREE = 0, DOF_DIR = 1, DOF_TIED = 2 };
// residual-form row kinds
enum { RROW_ID = 0, RROW_FREESLIP = 1, RROW_FRONT = 2, RROW_INNER = 3 };

// Outputs of one instance's solve (device memory, copied back by the host).
struct InstOut {
    int iter_now;
    int lin_iter;
    int lin_fail;
    int lim_n;
    double resid;
    double lin_resid;
    int status;        // YGPU_* of the solve
    int lin_status;    // status of the last linear solve
    int outer_iter;    // mixed: defect-correction steps
    int converged;
    int n_active;      // cells with a non-identity row (the Krylov iterations visit these)
    // state carried between the step kernels of the Picard loop
    int done;          // solve finished (converged, iteration limit or error)
    int in_alt;        // the current viscosity lives in visc_alt
    double bn2;        // ||b||^2 of this iteration's linear system
    int lin_it;        // last linear solve: iterations, status, outer steps, residual
    int lin_st;
    int lin_outer;
    double lin_rr;
    int defer;         // set by the host: a finished solve waits for the host (neff hook)
    int want_finish;   // the post step found the solve finished (deferred)
    double phase_ns[10];   // device time per phase: setup, strain, column, faces, system, krylov, epilogue,
                           // final, and the all-reduce share of the solve and of the Krylov phase
};

YG_DEV unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// Descriptor of one instance (device memory). Field pointers follow
// ygpu_fields; the rest is scratch that the host code carves for the solve.
struct Inst {
    int nx, ny, nz, n2, nu;
    int kind;                      // YGPU_KIND_*
    double dx, dy, n_glen;
    // solve velocity (SSA: ux_b/uy_b, DIVA: ux_bar/uy_bar)
    double *u_x, *u_y;
    // DIVA outputs
    double *ux3, *uy3, *ux_b, *uy_b, *ux_i, *uy_i, *duxdz, *duydz, *beta_eff;
    double *taub_x, *taub_y, *beta, *beta_x, *beta_y;
    double *visc, *visc_int, *err_x, *err_y;
    const int *mask_x, *mask_y;
    const double *c_bed, *f_slide, *taud_x, *taud_y, *taul_x, *taul_y;
    const double *H, *f_ice, *H_grnd, *f_grnd, *fg_x, *fg_y, *ATT, *zeta, *z_sl, *z_bed;
    // scratch, 3D
    double* visc_alt;
    double* attp;                  // A^(-1/n) at the quadrature nodes (4 x nz x n2), constant in a solve
    double* lvis;                  // log of the current viscosity (nz x n2)
    // scratch, 2D
    double *ux_nm1, *uy_nm1, *bm_x, *bm_y, *lk_x, *lk_y, *lr_x, *lr_y, *F2, *F2x, *F2y, *Nab;
    double *tbp_x, *tbp_y, *drag_x, *drag_y;
    // linear system (nu entries each)
    double *x, *b, *r, *p, *q, *z, *dinv, *rt, *v, *s, *t, *ph, *sh, *dval, *m2;
    int *ukind, *emap, *mem, *rpart;
    // cells with a non-identity row, in cell order (n2 + 1 ints; [n2] = count)
    int* acell;
    // per-cell flags of the solve's fixed inputs, set by the setup step (CF_*)
    unsigned char* cflag;
    // mixed precision scratch (nu entries; coefficient copies n2)
    float *fN, *fNab, *fdrag_x, *fdrag_y, *fdinv;
    float* fminv;                  // mixed, block preconditioner: inverse of each 4x4-cell tile block (32x32)
    float *fx, *fr, *fp, *fq, *fz, *frt, *fv, *fs, *ft, *fph, *fsh, *fm2;
    float4* fst;                   // mixed CG: per unknown the records (z, q, s, p), (x, r, u, w)
    // -p ilu on the residual form: ILU(0) factors in a six-colour ordering, per
    // unknown YG_ILU_W slots of packed columns (column | colour group << 28, -1
    // unused), the factor values in slot order and the inverse pivot; FP64 for
    // the FP64 solve, FP32 for the mixed inner solves
    int* icol;
    double *ilu, *ipiv;
    float *filu, *fipiv;
    InstOut* out;
    int visc_final_in_alt;         // set by the kernel: final visc is in visc_alt
};

#define YG_ILU_W 9                 // slots of an ILU(0) row of the residual form

// ---------------------------------------------------------------------------
// Team of CTAs: barrier and fused all-reduce (bounded waits)
// ---------------------------------------------------------------------------
#define YG_MAX_TEAM_CTAS 1024
#define YG_REC_MAX_CTAS 16         // teams up to this size poll the FP32 all-reduce records
#define YG_RED_MAX 4

// Team barrier: every CTA adds 1 to `count` with a release reduction and
// waits (one thread, acquire loads) until count reaches its target, which
// grows by the team's CTA count at each barrier. `base` holds count at the
// start of a launch (CTA 0 stores it at the end of the previous launch, after
// its last arrival; every CTA reads it before its first).
struct __align__(16) TeamCtl {
    unsigned int count;
    unsigned int base;
    int abort;
    int inst;                      // instance the team works on (work queue)
    unsigned int abase;            // generation of the last FP32 all-reduce of a launch (CTA 0
                                   // stores it at the end, every CTA reads it at the start)
    unsigned char spin_log2;       // 0: waits give up after YG_SPIN_LIMIT polls; k: after 2^k
    union __align__(16) {          // per-CTA totals of the all-reduces, by parity; the
                                   // YG_RED_MAX totals of a CTA are one 16/32-byte record
        double slots[2][YG_MAX_TEAM_CTAS][YG_RED_MAX];
        float fslots[2][YG_MAX_TEAM_CTAS][YG_RED_MAX];
    };
    // FP32 all-reduce records: per CTA YG_RED_MAX words (generation << 32 | FP32
    // bits), by parity; a word is read and written whole, so a reader that sees
    // the current generation in every word of a record has that CTA's totals
    unsigned long long rec[2][YG_MAX_TEAM_CTAS][YG_RED_MAX];
};
template <typename V>
YG_DEV V* team_slot(TeamCtl* c, int parity, int cta, int k);
template <>
YG_DEV double* team_slot<double>(TeamCtl* c, int parity, int cta, int k) { return &c->slots[parity][cta][k]; }
template <>
YG_DEV float* team_slot<float>(TeamCtl* c, int parity, int cta, int k) { return &c->fslots[parity][cta][k]; }
// One CTA's record of YG_RED_MAX totals in a single round trip (L2, bypassing L1)
YG_DEV void team_slot_load(TeamCtl* c, int parity, int cta, float v[YG_RED_MAX]) {
    const float4 r = __ldcg(reinterpret_cast<const float4*>(&c->fslots[parity][cta][0]));
    v[0] = r.x; v[1] = r.y; v[2] = r.z; v[3] = r.w;
}
YG_DEV void team_slot_load(TeamCtl* c, int parity, int cta, double v[YG_RED_MAX]) {
    const double2* p = reinterpret_cast<const double2*>(&c->slots[parity][cta][0]);
    const double2 r0 = __ldcg(p), r1 = __ldcg(p + 1);
    v[0] = r0.x; v[1] = r0.y; v[2] = r1.x; v[3] = r1.y;
}

struct Team {
    int cta, ncta;                 // rank of this CTA in the team, CTAs in the team
    int tid, nthr;                 // thread rank in the team, threads in the team
    int parity;                    // reduction slot buffer in use
    TeamCtl* ctl;
    int* abort_all;                // whole-launch abort flag (timeout anywhere)
    unsigned long long sync_ns;    // time thread 0 of the CTA spent in team all-reduces (ns; an
                                   // integer, so that the count adds nothing to the FP64 pipe)
    unsigned gen;                  // thread 0: count target of the last team barrier
    unsigned agen;                 // every thread: generation of the last FP32 all-reduce
    unsigned spin_lim;             // thread 0: polls after which a wait gives up
    bool cl;                       // the team is one thread-block cluster: barriers are the
                                   // hardware cluster barrier, all-reduces go through
                                   // distributed shared memory (no global control block)
};

// A register copy of the team for the body of a noinline solver. The caller's
// Team lives in its stack frame (local memory); the team barriers and
// all-reduces read and update its fields on every call from every thread, so
// the loops work on this copy, which is written back when the function returns.
struct TeamLocal {
    Team& ref;
    Team t;
    YG_DEV explicit TeamLocal(Team& r) : ref(r), t(r) {}
    YG_DEV ~TeamLocal() { ref = t; }
};

YG_DEV unsigned ld_acquire_u32(const unsigned int* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
YG_DEV int ld_acquire_s32(const int* p) {
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Spin budget of one barrier wait: 2^22 acquire polls of the L2 (about a
// second or more). A wait that runs out sets the abort flags; every later wait of the
// launch returns at once, and the kernel reports YGPU_ERR_TIMEOUT. The control
// block can lower the budget to 2^spin_log2 polls (ygpu_tuning.spin_log2, for tests
// of the timeout path).
#define YG_SPIN_LIMIT (1u << 22)
YG_DEV unsigned team_spin_limit(const TeamCtl* c) {
    const unsigned k = *(const volatile unsigned char*)&c->spin_log2;
    return (k == 0u || k > 22u) ? YG_SPIN_LIMIT : (1u << k);
}

YG_DEV void red_release_add_u32(unsigned int* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Returns false if the launch is aborting. The release reduction by thread 0
// follows a __syncthreads, so the CTA's earlier writes are ordered before its
// arrival; the closing __syncthreads orders the CTA's later reads after thread
// 0's acquire. Counts wrap: the comparison is on the signed difference.
YG_DEV bool team_barrier(Team& T) {
    if (T.cl) {
        // barrier.cluster arrive (release) / wait (acquire): every thread of the
        // cluster's CTAs; orders the CTAs' global and shared memory accesses
        cooperative_groups::this_cluster().sync();
        return true;
    }
    __syncthreads();
    __shared__ int s_ok;
    if (threadIdx.x == 0) {
        int ok = 1;
        if (T.ncta > 1) {
            T.gen += (unsigned)T.ncta;
            red_release_add_u32(&T.ctl->count, 1u);
            unsigned n = 0;
            while ((int)(ld_acquire_u32(&T.ctl->count) - T.gen) < 0) {
                ++n;
                if ((n & 1023u) == 0u || n >= T.spin_lim) {
                    if (ld_acquire_s32(T.abort_all)) { ok = 0; break; }
                    if (n >= T.spin_lim) {
                        atomicExch(T.abort_all, 1);
                        atomicExch(&T.ctl->abort, 1);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

template <typename V>
YG_DEV V warp_sum(V v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// All-reduce (sum) of nv <= YG_RED_MAX values over the team, deterministic
// for a fixed launch shape. Every thread passes its partials; every thread
// gets the totals. Also acts as a team barrier. Every level (warp, CTA, team)
// sums in the partials' type V: the FP32 partials of the mixed inner solves
// never touch the FP64 pipe, whose dependent-add latency on this part is about
// fourteen times FP32's and which would otherwise dominate the all-reduce.
template <typename V>
YG_DEV bool team_allreduce_impl(Team& T, const V* in, V* out, int nv) {
    __shared__ V s_red[32][YG_RED_MAX];
    __shared__ V s_tot[YG_RED_MAX];
    // cluster teams: per-CTA totals in this CTA's shared memory, double-buffered
    // by parity (a CTA rewrites a buffer only after the next cluster barrier, which
    // every CTA passes after its reads of that buffer)
    __shared__ V s_cl[2][YG_RED_MAX];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // the nv sums are reduced side by side (independent shuffle chains)
    V w[YG_RED_MAX];
#pragma unroll
    for (int k = 0; k < YG_RED_MAX; k++) w[k] = (k < nv) ? in[k] : V(0);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < YG_RED_MAX; k++) w[k] += __shfl_xor_sync(0xffffffffu, w[k], o);
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < YG_RED_MAX; k++) s_red[wid][k] = w[k];
    __syncthreads();
    // warp 0: the CTA's totals (all YG_RED_MAX slots, unused ones 0)
    auto cta_totals = [&](V t[YG_RED_MAX]) {
#pragma unroll
        for (int k = 0; k < YG_RED_MAX; k++) t[k] = (lane < nw) ? s_red[lane][k] : V(0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
#pragma unroll
            for (int k = 0; k < YG_RED_MAX; k++) t[k] += __shfl_xor_sync(0xffffffffu, t[k], o);
    };
    if (T.cl) {
        if (wid == 0) {
            V t[YG_RED_MAX];
            cta_totals(t);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) s_cl[T.parity][k] = t[k];
        }
        cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
        cl.sync();
        if (wid == 0) {
            // every CTA sums the CTA totals in the same order: identical results
            V a[YG_RED_MAX];
#pragma unroll
            for (int k = 0; k < YG_RED_MAX; k++) a[k] = V(0);
            for (int c = lane; c < T.ncta; c += 32) {
                const V* r = cl.map_shared_rank(&s_cl[T.parity][0], c);
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) a[k] += r[k];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) s_tot[k] = a[k];
        }
        T.parity ^= 1;
        __syncthreads();
        for (int k = 0; k < nv; k++) out[k] = s_tot[k];
        // no closing barrier: s_tot and s_red are next written after the next
        // call's first __syncthreads, which every thread passes after these reads
        return true;
    }
    if constexpr (sizeof(V) == sizeof(float)) {
        if (T.ncta > 1 && T.ncta <= YG_REC_MAX_CTAS) {
            // FP32 sums of a small global team: each CTA publishes its totals as words
            // carrying the all-reduce's generation (release pattern: fence, then
            // relaxed stores); warp 0 of every CTA polls the records themselves
            // until every word shows the generation (acquire pattern: relaxed
            // loads, then a fence). One L2 round trip after the last CTA's
            // record lands, where a counter barrier followed by reads of the
            // totals takes three. Larger teams use the counter barrier: with
            // every CTA polling every record, the few L2 lines holding them
            // become the bottleneck.
            __shared__ int s_rok;
            const unsigned g = ++T.agen;
            if (wid == 0) {
                V t[YG_RED_MAX];
                cta_totals(t);
                if (lane == 0) {
                    unsigned long long w[YG_RED_MAX];
#pragma unroll
                    for (int k = 0; k < YG_RED_MAX; k++)
                        w[k] = ((unsigned long long)g << 32) | (unsigned long long)__float_as_uint((float)t[k]);
                    unsigned long long* r = &T.ctl->rec[T.parity][T.cta][0];
                    asm volatile("fence.acq_rel.gpu;" ::: "memory");
                    asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(r), "l"(w[0]), "l"(w[1]) : "memory");
                    asm volatile("st.relaxed.gpu.global.v2.b64 [%0], {%1, %2};" ::"l"(r + 2), "l"(w[2]), "l"(w[3]) : "memory");
                }
                V a[YG_RED_MAX];
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) a[k] = V(0);
                int ok = 1;
                unsigned n = 0;
                for (int c0 = 0; c0 < T.ncta && ok; c0 += 32) {
                    const int c = c0 + lane;
                    bool have = (c >= T.ncta);
                    unsigned long long w0 = 0, w1 = 0, w2 = 0, w3 = 0;
                    const unsigned long long* r = &T.ctl->rec[T.parity][c < T.ncta ? c : 0][0];
                    while (true) {
                        if (!have) {
                            asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(w0), "=l"(w1) : "l"(r) : "memory");
                            asm volatile("ld.relaxed.gpu.global.v2.b64 {%0, %1}, [%2];" : "=l"(w2), "=l"(w3) : "l"(r + 2) : "memory");
                            have = (unsigned)(w0 >> 32) == g && (unsigned)(w1 >> 32) == g && (unsigned)(w2 >> 32) == g &&
                                   (unsigned)(w3 >> 32) == g;
                        }
                        if (__all_sync(0xffffffffu, have)) break;
                        ++n;
                        if ((n & 1023u) == 0u || n >= T.spin_lim) {
                            int ab = ld_acquire_s32(T.abort_all);
                            if (!ab && n >= T.spin_lim && lane == 0) {
                                atomicExch(T.abort_all, 1);
                                atomicExch(&T.ctl->abort, 1);
                            }
                            ab = __shfl_sync(0xffffffffu, ab, 0);
                            if (ab || n >= T.spin_lim) { ok = 0; break; }
                        }
                    }
                    if (ok && c < T.ncta) {
                        a[0] += __uint_as_float((unsigned)w0);
                        a[1] += __uint_as_float((unsigned)w1);
                        a[2] += __uint_as_float((unsigned)w2);
                        a[3] += __uint_as_float((unsigned)w3);
                    }
                }
                asm volatile("fence.acq_rel.gpu;" ::: "memory");
#pragma unroll
                for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                    for (int k = 0; k < YG_RED_MAX; k++) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
                if (lane == 0) {
#pragma unroll
                    for (int k = 0; k < YG_RED_MAX; k++) s_tot[k] = a[k];
                    s_rok = ok;
                }
            }
            T.parity ^= 1;
            __syncthreads();
            for (int k = 0; k < nv; k++) out[k] = s_tot[k];
            return s_rok != 0;
        }
    }
    if (wid == 0) {
        V t[YG_RED_MAX];
        cta_totals(t);
        if (lane == 0) {
            if (T.ncta > 1) {
                V* r = team_slot<V>(T.ctl, T.parity, T.cta, 0);
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) r[k] = t[k];
            } else {
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) s_tot[k] = t[k];
            }
        }
    }
    if (T.ncta > 1) {
        if (!team_barrier(T)) return false;
        if (wid == 0) {
            // one record (all the sums of a CTA) per load: a single L2 round trip
            // for teams of up to 32 CTAs
            V a[YG_RED_MAX];
#pragma unroll
            for (int k = 0; k < YG_RED_MAX; k++) a[k] = V(0);
            for (int c = lane; c < T.ncta; c += 32) {
                V r[YG_RED_MAX];
                team_slot_load(T.ctl, T.parity, c, r);
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) a[k] += r[k];
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) a[k] += __shfl_xor_sync(0xffffffffu, a[k], o);
            if (lane == 0)
#pragma unroll
                for (int k = 0; k < YG_RED_MAX; k++) s_tot[k] = a[k];
        }
        T.parity ^= 1;
    }
    __syncthreads();
    for (int k = 0; k < nv; k++) out[k] = s_tot[k];
    // no closing barrier (see the cluster branch)
    return true;
}
template <typename V>
YG_DEV bool team_allreduce_w(Team& T, const V* in, V* out, int nv) {
    const unsigned long long t0 = (threadIdx.x == 0) ? global_ns() : 0ull;
    bool ok = team_allreduce_impl<V>(T, in, out, nv);
    if (threadIdx.x == 0) T.sync_ns += global_ns() - t0;
    return ok;
}
YG_DEV bool team_allreduce(Team& T, double* vals, int nv) { return team_allreduce_w<double>(T, vals, vals, nv); }

// Exclusive prefix sums over the team's CTAs, in CTA rank order, of nv <=
// YG_RED_MAX per-CTA values held by thread 0 (exact for integers below 2^53),
// and their totals; every thread gets both. Also acts as a team barrier.
YG_DEV bool team_scan_cta(Team& T, const double* mine, double* before, double* total, int nv) {
    __shared__ double s_b[YG_RED_MAX], s_t[YG_RED_MAX];
    if (T.ncta == 1) {
        if (threadIdx.x == 0)
            for (int k = 0; k < nv; k++) { s_b[k] = 0.0; s_t[k] = mine[k]; }
    } else {
        if (threadIdx.x == 0)
            for (int k = 0; k < nv; k++) T.ctl->slots[T.parity][T.cta][k] = mine[k];
        if (!team_barrier(T)) return false;
        if (threadIdx.x < 32) {
            const int lane = threadIdx.x;
            for (int k = 0; k < nv; k++) {
                double wb = 0.0, wt = 0.0;
                for (int c = lane; c < T.ncta; c += 32) {
                    const double v = __ldcg(&T.ctl->slots[T.parity][c][k]);
                    wt += v;
                    if (c < T.cta) wb += v;
                }
                wb = warp_sum<double>(wb);
                wt = warp_sum<double>(wt);
                if (lane == 0) { s_b[k] = wb; s_t[k] = wt; }
            }
        }
        T.parity ^= 1;
    }
    __syncthreads();
    for (int k = 0; k < nv; k++) { before[k] = s_b[k]; total[k] = s_t[k]; }
    __syncthreads();
    return true;
}

// Integer all-reduce helpers via the double path (exact for |v| < 2^53).
YG_DEV bool team_allreduce_or_max(Team& T, double* vals, int nv) { return team_allreduce(T, vals, nv); }
