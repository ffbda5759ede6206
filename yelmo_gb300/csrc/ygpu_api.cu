// ygpu_api.cu -- C ABI of libyelmo_gpu.so: parameter helpers, contexts,
// device-resident solves, and the host-pointer drop-ins for
// calc_velocity_ssa / calc_velocity_diva / set_ssa_masks / the calc_ydyn
// prologue / linear_solver_matrix_solve.
#include <cuda_runtime.h>

#include <math.h>
#include <stdarg.h>
#include <stddef.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <queue>
#include <thread>
#include <utility>
#include <numeric>
#include <vector>

#include "ygpu_common.cuh"
#include "ygpu_host.h"

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local std::string t_err;

void ygpu_set_error(const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    t_err = buf;
}

#define CK(call)                                                                         \
    do {                                                                                 \
        cudaError_t e_ = (call);                                                         \
        if (e_ != cudaSuccess) {                                                         \
            ygpu_set_error("%s:%d %s: %s", __FILE__, __LINE__, #call, cudaGetErrorString(e_)); \
            return YGPU_ERR_CUDA;                                                        \
        }                                                                                \
    } while (0)

extern "C" const char* ygpu_last_error(void) { return t_err.c_str(); }
extern "C" const char* ygpu_version(void) { return "yelmo_gb300 0.1 (sm_103a)"; }

// ---------------------------------------------------------------------------
// parameters
// ---------------------------------------------------------------------------
extern "C" void ygpu_dyn_par_defaults(ygpu_dyn_par* p) {
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
    p->precision = YGPU_PREC_FP64;
}

extern "C" int ygpu_parse_lis_opt(const char* opts, ygpu_dyn_par* p) {
    if (!opts || !p) return YGPU_ERR_BAD_ARG;
    std::vector<std::string> tok;
    const char* s = opts;
    while (*s) {
        while (*s == ' ' || *s == '\t') s++;
        const char* e = s;
        while (*e && *e != ' ' && *e != '\t') e++;
        if (e > s) tok.emplace_back(s, e - s);
        s = e;
    }
    if (tok.size() % 2) {
        ygpu_set_error("LIS option string has an option without value: %s", opts);
        return YGPU_ERR_BAD_ARG;
    }
    for (size_t k = 0; k < tok.size(); k += 2) {
        const std::string& key = tok[k];
        const std::string& v = tok[k + 1];
        if (key == "-i") {
            if (v == "cg" || v == "1") p->lin_solver = YGPU_LIN_CG;
            else if (v == "bicgstab" || v == "3") p->lin_solver = YGPU_LIN_BICGSTAB;
            else if (v == "minres" || v == "5") p->lin_solver = YGPU_LIN_MINRES;
            else { ygpu_set_error("LIS solver not supported: %s", v.c_str()); return YGPU_ERR_BAD_ARG; }
        } else if (key == "-p") {
            if (v == "none" || v == "0") p->lin_precond = YGPU_PRE_NONE;
            else if (v == "jacobi" || v == "1") p->lin_precond = YGPU_PRE_JACOBI;
            else if (v == "ilu" || v == "2") p->lin_precond = YGPU_PRE_ILU0;
            else { ygpu_set_error("LIS preconditioner not supported: %s", v.c_str()); return YGPU_ERR_BAD_ARG; }
        } else if (key == "-maxiter") {
            p->lin_maxiter = atoi(v.c_str());
        } else if (key == "-tol") {
            p->lin_tol = atof(v.c_str());
        } else if (key == "-initx_zeros") {
            p->lin_initx_zeros = (v == "true" || v == "1");
        }
    }
    return YGPU_OK;
}

extern "C" int ygpu_boundary_code(const char* b) {
    if (!b) return -1;
    if (!strcmp(b, "zeros")) return YGPU_BND_ZEROS;
    if (!strcmp(b, "infinite") || !strcmp(b, "mask")) return YGPU_BND_INFINITE;
    if (!strcmp(b, "MISMIP3D")) return YGPU_BND_MISMIP3D;
    if (!strcmp(b, "TROUGH")) return YGPU_BND_TROUGH;
    if (!strcmp(b, "periodic")) return YGPU_BND_PERIODIC;
    if (!strcmp(b, "periodic-x")) return YGPU_BND_PERIODIC_X;
    if (!strcmp(b, "periodic-y")) return YGPU_BND_PERIODIC_Y;
    return -1;
}

int ygpu_check_par(const ygpu_dyn_par* p) {
    if (!p) { ygpu_set_error("par is NULL"); return YGPU_ERR_BAD_ARG; }
    if (p->boundaries < 0 || p->boundaries > 6) { ygpu_set_error("bad boundary code %d", p->boundaries); return YGPU_ERR_BAD_ARG; }
    if (p->visc_method < 0 || p->visc_method > 2) { ygpu_set_error("visc_method not recognized: %d", p->visc_method); return YGPU_ERR_BAD_ARG; }
    if (p->beta_method < -1 || p->beta_method > 5) { ygpu_set_error("beta_method not recognized: %d", p->beta_method); return YGPU_ERR_BAD_ARG; }
    if (p->beta_gl_stag < -1 || p->beta_gl_stag > 4) { ygpu_set_error("beta_gl_stag not recognized: %d", p->beta_gl_stag); return YGPU_ERR_BAD_ARG; }
    if (p->beta_gl_scale < 0 || p->beta_gl_scale > 3) { ygpu_set_error("beta_gl_scale not recognized: %d", p->beta_gl_scale); return YGPU_ERR_BAD_ARG; }
    if (p->beta_gl_scale == 0 && (p->beta_gl_f < 0.0 || p->beta_gl_f > 1.0)) { ygpu_set_error("beta_gl_f must be between 0 and 1"); return YGPU_ERR_BAD_ARG; }
    if (p->beta_gl_scale == 1 && p->H_grnd_lim <= 0.0) { ygpu_set_error("H_grnd_lim must be positive"); return YGPU_ERR_BAD_ARG; }
    if (p->ssa_solver != YGPU_SSA_RESIDUAL && p->ssa_solver != YGPU_SSA_ENERGY) { ygpu_set_error("bad ssa_solver"); return YGPU_ERR_BAD_ARG; }
    if (p->ssa_iter_max < 0 || p->lin_maxiter < 0) { ygpu_set_error("negative iteration limit"); return YGPU_ERR_BAD_ARG; }
    if (!(p->ssa_vel_max > 0.0)) { ygpu_set_error("ssa_vel_max must be positive"); return YGPU_ERR_BAD_ARG; }
    return YGPU_OK;
}

// ---------------------------------------------------------------------------
// context
// ---------------------------------------------------------------------------
struct ygpu_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    char* arena = nullptr;          // per-instance scratch
    size_t arena_cap = 0;
    char* fbuf = nullptr;           // fields of host-pointer calls
    size_t fbuf_cap = 0;
    char* hbuf = nullptr;           // pinned host mirror of fbuf
    size_t hbuf_cap = 0;
    char* dpieces = nullptr;        // copy list of the direct host<->device copies
    size_t dpieces_cap = 0;
    int pageable = -1;              // the device reads and writes pageable host memory (-1: not asked yet)
    Inst* d_insts = nullptr;
    int insts_cap = 0;
    InstOut* d_out = nullptr;
    int out_cap = 0;
    TeamCtl* d_ctl = nullptr;
    int ctl_cap = 0;
    int* d_map = nullptr;           // team plan of a batch (ygpu_plan_teams)
    int map_cap = 0;
    GraphCache graph;               // chunk graph of the last launch shape
    bool use_graphs = true;
    int check_every = 4;            // Picard iterations between host checks
    std::vector<double> hook_buf;   // host buffers of the neff hook
    int unknowns_per_cta = 0;       // team size: unknowns per CTA (0: 2 x block)
    size_t max_active_unknowns = 1500000;   // batches beyond this run as a queue (continuous batching)
    int spin_log2 = 0;              // team waits give up after 2^spin_log2 polls (0: the default 2^22)
    int cluster_ctas = 0;           // Krylov cluster teams of this many CTAs (2..16; else off)
    int* h_flags = nullptr;         // pinned: finished count, abort flag
    int* d_misc = nullptr;          // [0] queue, [1] abort, [2..3] csr out
    double* d_miscd = nullptr;
    int max_ctas = 0;
    int csr_max_ctas = 0;
    int adv_max_ctas = 0;
    int sms = 0;
    std::vector<Inst> h_insts;
    std::vector<InstOut> h_out;
};

static int grow(char** p, size_t* cap, size_t need) {
    if (*cap >= need) return YGPU_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc((void**)p, need) != cudaSuccess) {
        cudaGetLastError();
        ygpu_set_error("device allocation of %zu bytes failed", need);
        return YGPU_ERR_NOMEM;
    }
    *cap = need;
    return YGPU_OK;
}

extern "C" void ygpu_tuning_defaults(ygpu_tuning* t) {
    if (!t) return;
    t->check_every = 4;
    t->use_graphs = 1;
    t->unknowns_per_cta = 2 * YG_BLOCK;
    t->max_active_unknowns = 1500000;
    t->spin_log2 = 0;
    t->cluster_ctas = 0;
}

extern "C" int ygpu_ctx_set_tuning(ygpu_ctx* c, const ygpu_tuning* t) {
    if (!c || !t) { ygpu_set_error("NULL argument"); return YGPU_ERR_BAD_ARG; }
    if (t->check_every < 1 || t->check_every > 64 || t->unknowns_per_cta < 32 || t->unknowns_per_cta > (1 << 20) ||
        t->spin_log2 < 0 || t->spin_log2 > 22 || t->cluster_ctas < -1 || t->cluster_ctas == 1 || t->cluster_ctas > 16) {
        ygpu_set_error("tuning out of range: check_every %d (1..64), unknowns_per_cta %d (32..2^20), spin_log2 %d "
                       "(0..22), cluster_ctas %d (-1, 0, 2..16)", t->check_every, t->unknowns_per_cta, t->spin_log2,
                       t->cluster_ctas);
        return YGPU_ERR_BAD_ARG;
    }
    c->check_every = t->check_every;
    c->use_graphs = (t->use_graphs != 0);
    c->unknowns_per_cta = t->unknowns_per_cta;
    c->max_active_unknowns = t->max_active_unknowns;
    c->spin_log2 = t->spin_log2;
    c->cluster_ctas = t->cluster_ctas;
    ygpu_graph_cache_clear(&c->graph);
    return YGPU_OK;
}

extern "C" ygpu_ctx* ygpu_ctx_create(int device) {
    ygpu_ctx* c = new ygpu_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->e0) != cudaSuccess || cudaEventCreate(&c->e1) != cudaSuccess ||
        cudaMalloc((void**)&c->d_misc, 64) != cudaSuccess || cudaMalloc((void**)&c->d_miscd, 64) != cudaSuccess ||
        cudaMallocHost((void**)&c->h_flags, 2 * sizeof(int)) != cudaSuccess) {
        ygpu_set_error("context creation on device %d failed: %s", device, cudaGetErrorString(cudaGetLastError()));
        delete c;
        return nullptr;
    }
    // the step kernels' non-inlined phases take up to about 1.3 KB of stack per
    // thread (ptxas' cumulative stack size), above the default limit: give them 4 KB
    size_t stack = 0;
    cudaDeviceGetLimit(&stack, cudaLimitStackSize);
    if (stack < 4096) cudaDeviceSetLimit(cudaLimitStackSize, 4096);
    c->max_ctas = ygpu_solver_max_ctas(device);
    c->csr_max_ctas = ygpu_csr_max_ctas(device);
    c->adv_max_ctas = ygpu_adv_max_ctas(device);
    c->sms = ygpu_sm_count(device);
    return c;
}

extern "C" void ygpu_ctx_destroy(ygpu_ctx* c) {
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    cudaFree(c->arena);
    cudaFree(c->fbuf);
    if (c->dpieces) cudaFree(c->dpieces);
    if (c->hbuf) cudaFreeHost(c->hbuf);
    cudaFree(c->d_insts);
    cudaFree(c->d_out);
    cudaFree(c->d_ctl);
    cudaFree(c->d_map);
    ygpu_graph_cache_clear(&c->graph);
    if (c->h_flags) cudaFreeHost(c->h_flags);
    cudaFree(c->d_misc);
    cudaFree(c->d_miscd);
    if (c->e0) cudaEventDestroy(c->e0);
    if (c->e1) cudaEventDestroy(c->e1);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

extern "C" void* ygpu_ctx_stream(ygpu_ctx* c) { return c ? (void*)c->stream : nullptr; }

// neff hook of the calling thread (DIVA single solves)
static thread_local ygpu_neff_hook t_hook = nullptr;
static thread_local void* t_hook_user = nullptr;
extern "C" void ygpu_set_neff_hook(ygpu_neff_hook hook, void* user) {
    t_hook = hook;
    t_hook_user = hook ? user : nullptr;
}
bool ygpu_neff_hook_is_set() { return t_hook != nullptr; }

// The method and preconditioner linear_solve (ygpu_solver.cu) runs for a
// parameter set: CG on the energy form unless BiCGSTAB is asked for, BiCGSTAB
// on the residual form; "-p ilu" is ILU(0) (six-colour ordering) with BiCGSTAB
// on the residual form, the tile block preconditioner with CG on the energy
// form, and Jacobi with BiCGSTAB on the energy form. nx, ny > 0: the grid of the
// solve, whose periodic directions the ILU(0) colouring needs in multiples of 3
// (Jacobi otherwise).
void ygpu_lin_method_run_grid(const ygpu_dyn_par* p, int nx, int ny, int* solver, int* precond) {
    if (!p) return;
    const bool energy = (p->ssa_solver == YGPU_SSA_ENERGY);
    const bool cg = energy && p->lin_solver != YGPU_LIN_BICGSTAB;
    int pc = p->lin_precond;
    if (pc == YGPU_PRE_ILU0) {
        if (cg) pc = YGPU_PRE_TILE_BLOCK;
        else if (energy) pc = YGPU_PRE_JACOBI;
        else if (nx > 0 && ny > 0 && !ygpu_ilu_colourable(nx, ny, p->boundaries)) pc = YGPU_PRE_JACOBI;
    }
    if (solver) *solver = cg ? YGPU_LIN_CG : YGPU_LIN_BICGSTAB;
    if (precond) *precond = pc;
}
extern "C" void ygpu_lin_method_run(const ygpu_dyn_par* p, int* solver, int* precond) {
    ygpu_lin_method_run_grid(p, 0, 0, solver, precond);
}

// default context of the calling thread (host-pointer entry points)
static thread_local ygpu_ctx* t_ctx = nullptr;
static ygpu_ctx* default_ctx() {
    int dev = 0;
    cudaGetDevice(&dev);
    if (t_ctx && t_ctx->device != dev) {
        ygpu_ctx_destroy(t_ctx);
        t_ctx = nullptr;
    }
    if (!t_ctx) t_ctx = ygpu_ctx_create(dev);
    return t_ctx;
}

// ---------------------------------------------------------------------------
// scratch layout of one instance
// ---------------------------------------------------------------------------
size_t ygpu_align256(size_t b) { return (b + 255) & ~(size_t)255; }
static size_t al(size_t b) { return ygpu_align256(b); }

static size_t tile_blocks(int nx, int ny) { return (size_t)((nx + 3) / 4) * ((ny + 3) / 4); }

size_t ygpu_inst_scratch_bytes(int nx, int ny, int nz, bool mixed, bool block, bool ilu) {
    size_t n2 = (size_t)nx * ny, nu = 2 * n2, n3 = n2 * nz;
    size_t b = al(n3 * 8);               // visc_alt
    b += al(4 * n3 * 8) + al(n3 * 8);    // attp, lvis
    b += 16 * al(n2 * 8);                // 2D scratch
    b += 15 * al(nu * 8);                // linear system
    b += 6 * al(nu * 4);                 // ukind, emap, mem(3), rpart
    b += al((n2 + 1) * 4);               // active cell list
    b += al(n2);                         // cell flags
    if (mixed) b += 4 * al(n2 * 4) + 13 * al(nu * 4) + al(8 * nu * 4);   // + CG row records
    if (block) b += al(tile_blocks(nx, ny) * 1024 * 4);
    if (ilu) b += al(YG_ILU_W * nu * 4) + al(YG_ILU_W * nu * 8) + al(nu * 8);   // FP64 factors in both modes
    return b;
}

void ygpu_inst_scratch_carve(Inst& I, char* base, int nx, int ny, int nz, bool mixed, bool block, bool ilu) {
    size_t n2 = (size_t)nx * ny, nu = 2 * n2, n3 = n2 * nz;
    char* p = base;
    auto D = [&](size_t n) { double* r = (double*)p; p += al(n * 8); return r; };
    auto Iv = [&](size_t n) { int* r = (int*)p; p += al(n * 4); return r; };
    auto Fv = [&](size_t n) { float* r = (float*)p; p += al(n * 4); return r; };
    I.visc_alt = D(n3);
    I.attp = D(4 * n3);
    I.lvis = D(n3);
    I.ux_nm1 = D(n2); I.uy_nm1 = D(n2); I.bm_x = D(n2); I.bm_y = D(n2);
    I.lk_x = D(n2); I.lk_y = D(n2); I.lr_x = D(n2); I.lr_y = D(n2);
    I.F2 = D(n2); I.F2x = D(n2); I.F2y = D(n2); I.Nab = D(n2);
    I.tbp_x = D(n2); I.tbp_y = D(n2); I.drag_x = D(n2); I.drag_y = D(n2);
    I.x = D(nu); I.b = D(nu); I.r = D(nu); I.p = D(nu); I.q = D(nu); I.z = D(nu); I.dinv = D(nu);
    I.rt = D(nu); I.v = D(nu); I.s = D(nu); I.t = D(nu); I.ph = D(nu); I.sh = D(nu); I.dval = D(nu);
    I.m2 = D(nu);
    I.ukind = Iv(nu); I.emap = Iv(nu); I.mem = Iv(3 * nu); I.rpart = Iv(nu);
    I.acell = Iv(n2 + 1);
    I.cflag = (unsigned char*)p;
    p += al(n2);
    if (mixed) {
        I.fN = Fv(n2); I.fNab = Fv(n2); I.fdrag_x = Fv(n2); I.fdrag_y = Fv(n2);
        I.fdinv = Fv(nu); I.fx = Fv(nu); I.fr = Fv(nu); I.fp = Fv(nu); I.fq = Fv(nu); I.fz = Fv(nu);
        I.frt = Fv(nu); I.fv = Fv(nu); I.fs = Fv(nu); I.ft = Fv(nu); I.fph = Fv(nu); I.fsh = Fv(nu);
        I.fm2 = Fv(nu);
        I.fst = (float4*)Fv(8 * nu);
    } else {
        I.fst = nullptr;
        I.fN = I.fNab = I.fdrag_x = I.fdrag_y = I.fdinv = nullptr;
        I.fx = I.fr = I.fp = I.fq = I.fz = I.frt = I.fv = I.fs = I.ft = I.fph = I.fsh = I.fm2 = nullptr;
    }
    I.fminv = block ? Fv(tile_blocks(nx, ny) * 1024) : nullptr;
    I.icol = ilu ? Iv(YG_ILU_W * nu) : nullptr;
    I.ilu = I.ipiv = nullptr;
    I.filu = I.fipiv = nullptr;
    if (ilu) {
        // -p ilu runs on the residual form, whose BiCGSTAB is FP64 in both modes
        I.ilu = D(YG_ILU_W * nu);
        I.ipiv = D(nu);
    }
}

int ygpu_fields_check(int kind, const ygpu_fields* f) {
    if (!f) { ygpu_set_error("fields is NULL"); return YGPU_ERR_BAD_ARG; }
    if (f->nx < 3 || f->ny < 3 || f->nz < 2) {
        ygpu_set_error("grid too small: nx=%d ny=%d nz=%d (need nx,ny >= 3, nz >= 2)", f->nx, f->ny, f->nz);
        return YGPU_ERR_BAD_ARG;
    }
    if ((size_t)f->nx * f->ny > (size_t)(1 << 29)) { ygpu_set_error("grid too large"); return YGPU_ERR_BAD_ARG; }
    if (!(f->dx > 0.0) || !(f->dy > 0.0) || !(f->n_glen > 0.0)) { ygpu_set_error("dx, dy and n_glen must be positive"); return YGPU_ERR_BAD_ARG; }
    const void* need[] = {f->taub_acx, f->taub_acy, f->beta, f->beta_acx, f->beta_acy, f->visc_eff, f->visc_eff_int,
                          f->ssa_err_acx, f->ssa_err_acy, f->ssa_mask_acx, f->ssa_mask_acy, f->c_bed, f->f_slide,
                          f->taud_acx, f->taud_acy, f->taul_int_acx, f->taul_int_acy, f->H_ice, f->f_ice, f->H_grnd,
                          f->f_grnd, f->f_grnd_acx, f->f_grnd_acy, f->ATT, f->zeta_aa, f->z_sl, f->z_bed,
                          f->ux_b, f->uy_b};
    for (const void* q : need)
        if (!q) { ygpu_set_error("a required field pointer is NULL"); return YGPU_ERR_BAD_ARG; }
    if (kind == YGPU_KIND_DIVA) {
        const void* nd[] = {f->ux, f->uy, f->ux_bar, f->uy_bar, f->ux_i, f->uy_i, f->beta_eff, f->duxdz, f->duydz};
        for (const void* q : nd)
            if (!q) { ygpu_set_error("a DIVA field pointer is NULL"); return YGPU_ERR_BAD_ARG; }
    }
    return YGPU_OK;
}

void ygpu_fill_inst(Inst& I, int kind, const ygpu_fields* f) {
    memset(&I, 0, sizeof(I));
    I.nx = f->nx; I.ny = f->ny; I.nz = f->nz; I.n2 = f->nx * f->ny; I.nu = 2 * I.n2;
    I.kind = kind;
    I.dx = f->dx; I.dy = f->dy; I.n_glen = f->n_glen;
    if (kind == YGPU_KIND_DIVA) {
        I.u_x = f->ux_bar; I.u_y = f->uy_bar;
        I.ux3 = f->ux; I.uy3 = f->uy; I.ux_i = f->ux_i; I.uy_i = f->uy_i;
        I.duxdz = f->duxdz; I.duydz = f->duydz; I.beta_eff = f->beta_eff;
    } else {
        I.u_x = f->ux_b; I.u_y = f->uy_b;
    }
    I.ux_b = f->ux_b; I.uy_b = f->uy_b;
    I.taub_x = f->taub_acx; I.taub_y = f->taub_acy;
    I.beta = f->beta; I.beta_x = f->beta_acx; I.beta_y = f->beta_acy;
    I.visc = f->visc_eff; I.visc_int = f->visc_eff_int;
    I.err_x = f->ssa_err_acx; I.err_y = f->ssa_err_acy;
    I.mask_x = f->ssa_mask_acx; I.mask_y = f->ssa_mask_acy;
    I.c_bed = f->c_bed; I.f_slide = f->f_slide;
    I.taud_x = f->taud_acx; I.taud_y = f->taud_acy; I.taul_x = f->taul_int_acx; I.taul_y = f->taul_int_acy;
    I.H = f->H_ice; I.f_ice = f->f_ice; I.H_grnd = f->H_grnd; I.f_grnd = f->f_grnd;
    I.fg_x = f->f_grnd_acx; I.fg_y = f->f_grnd_acy; I.ATT = f->ATT; I.zeta = f->zeta_aa;
    I.z_sl = f->z_sl; I.z_bed = f->z_bed;
}

int ygpu_single_team_ctas(int max_ctas, size_t nu, int unknowns_per_cta) {
    const int upc = unknowns_per_cta > 0 ? unknowns_per_cta : 2 * YG_BLOCK;
    int tc = (int)((nu + upc - 1) / upc);
    if (tc < 1) tc = 1;
    if (tc > max_ctas) tc = max_ctas;
    if (tc > YG_MAX_TEAM_CTAS) tc = YG_MAX_TEAM_CTAS;
    return tc;
}


// Launch shape of a batch: (n_teams, team_ctas).
void ygpu_choose_teams(int max_ctas, int n_inst, size_t max_nu, int* n_teams, int* team_ctas, int upc) {
    int maxc = max_ctas > 0 ? max_ctas : 1;
    if (n_inst == 1) {
        // one team over the GPU, sized to the instance
        *team_ctas = ygpu_single_team_ctas(maxc, max_nu, upc);
        *n_teams = 1;
        return;
    }
    // teams share the GPU: as many CTAs per team as the batch leaves, but no more
    // than one CTA per ~4096 unknowns of the largest instance
    int auto_tc = maxc / n_inst;
    int by_size = (int)(max_nu / 4096);
    if (auto_tc > by_size) auto_tc = by_size;
    if (auto_tc < 1) auto_tc = 1;
    int tc = auto_tc;
    if (tc > maxc) tc = maxc;
    if (tc > YG_MAX_TEAM_CTAS) tc = YG_MAX_TEAM_CTAS;
    int nt = maxc / tc;
    if (nt > n_inst) nt = n_inst;
    if (nt < 1) nt = 1;
    *team_ctas = tc;
    *n_teams = nt;
}

bool ygpu_plan_teams(int max_ctas, int n, const size_t* nu, std::vector<int>& map, int* grid, int upc) {
    if (n < 1 || n > max_ctas) return false;
    std::vector<int> cnt(n, 1), cap(n);
    for (int q = 0; q < n; q++) cap[q] = ygpu_single_team_ctas(max_ctas, nu[q], upc);
    // greedy: the next CTA goes to the instance with the most unknowns per CTA
    std::priority_queue<std::pair<double, int>> pq;
    for (int q = 0; q < n; q++)
        if (cnt[q] < cap[q]) pq.push({(double)nu[q] / cnt[q], q});
    int left = max_ctas - n;
    while (left > 0 && !pq.empty()) {
        const int q = pq.top().second;
        pq.pop();
        cnt[q]++;
        left--;
        if (cnt[q] < cap[q]) pq.push({(double)nu[q] / cnt[q], q});
    }
    int g = 0;
    for (int q = 0; q < n; q++) g += cnt[q];
    map.assign((size_t)g + 2 * (size_t)n, -1);
    int first = 0;
    for (int q = 0; q < n; q++) {
        for (int k = 0; k < cnt[q]; k++) map[first + k] = q;
        map[g + 2 * q] = first;
        map[g + 2 * q + 1] = cnt[q];
        first += cnt[q];
    }
    *grid = g;
    return true;
}

static int solve_batch(ygpu_ctx* c, int kind, const ygpu_dyn_par* par, int n, const ygpu_fields* inst,
                       ygpu_stats* stats, double* host_cbed = nullptr) {
    YgRange range("ygpu solve_batch");
    int st = ygpu_check_par(par);
    if (st) return st;
    if (kind != YGPU_KIND_SSA && kind != YGPU_KIND_DIVA) { ygpu_set_error("bad solver kind %d", kind); return YGPU_ERR_BAD_ARG; }
    if (n < 1) { ygpu_set_error("no instances"); return YGPU_ERR_BAD_ARG; }
    for (int k = 0; k < n; k++)
        if ((st = ygpu_fields_check(kind, &inst[k]))) return st;
    CK(cudaSetDevice(c->device));
    const bool mixed = (par->precision == YGPU_PREC_MIXED);
    std::vector<size_t> off(n);
    size_t total = 0, max_nu = 0;
    for (int k = 0; k < n; k++) {
        off[k] = total;
        total += al(ygpu_inst_scratch_bytes(inst[k].nx, inst[k].ny, inst[k].nz, mixed, ygpu_wants_block(*par),
                                              ygpu_wants_ilu(*par)));
        max_nu = std::max(max_nu, (size_t)2 * inst[k].nx * inst[k].ny);
    }
    if ((st = grow(&c->arena, &c->arena_cap, total))) return st;
    if (c->insts_cap < n) {
        cudaFree(c->d_insts);
        cudaFree(c->d_out);
        c->d_insts = nullptr;
        c->d_out = nullptr;
        CK(cudaMalloc((void**)&c->d_insts, sizeof(Inst) * (size_t)n));
        CK(cudaMalloc((void**)&c->d_out, sizeof(InstOut) * (size_t)n));
        c->insts_cap = n;
    }
    int n_teams, team_ctas;
    ygpu_choose_teams(c->max_ctas, n, max_nu, &n_teams, &team_ctas, c->unknowns_per_cta);
    // queue order: largest instance first (longest-processing-time first)
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (size_t)inst[a].nx * inst[a].ny * inst[a].nz > (size_t)inst[b].nx * inst[b].ny * inst[b].nz;
    });
    // uneven batches that fit the GPU at once: one team per instance, CTAs in
    // proportion to its unknowns
    std::vector<size_t> nus(n);
    for (int q = 0; q < n; q++) nus[q] = (size_t)2 * inst[order[q]].nx * inst[order[q]].ny;
    std::vector<int> map;
    int map_grid = 0;
    const bool mapped = n > 1 && ygpu_plan_teams(c->max_ctas, n, nus.data(), map, &map_grid, c->unknowns_per_cta);
    const int n_ctl = mapped ? n : n_teams;
    if (c->ctl_cap < n_ctl) {
        cudaFree(c->d_ctl);
        c->d_ctl = nullptr;
        CK(cudaMalloc((void**)&c->d_ctl, sizeof(TeamCtl) * (size_t)n_ctl));
        c->ctl_cap = n_ctl;
    }
    if (mapped && c->map_cap < (int)map.size()) {
        cudaFree(c->d_map);
        c->d_map = nullptr;
        CK(cudaMalloc((void**)&c->d_map, sizeof(int) * map.size()));
        c->map_cap = (int)map.size();
    }
    if (mapped)
        CK(cudaMemcpyAsync(c->d_map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, c->stream));
    c->h_insts.resize(n);
    for (int q = 0; q < n; q++) {
        const int k = order[q];
        Inst& I = c->h_insts[q];
        ygpu_fill_inst(I, kind, &inst[k]);
        ygpu_inst_scratch_carve(I, c->arena + off[k], inst[k].nx, inst[k].ny, inst[k].nz, mixed,
                                ygpu_wants_block(*par), ygpu_wants_ilu(*par));
        I.out = c->d_out + k;      // outputs stay in caller order
    }
    CK(cudaMemcpyAsync(c->d_insts, c->h_insts.data(), sizeof(Inst) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
    CK(cudaMemsetAsync(c->d_out, 0, sizeof(InstOut) * (size_t)n, c->stream));
    // neff hook of the calling thread: single DIVA solves, one iteration at a time
    NeffRun hr;
    const bool hooked = (t_hook && kind == YGPU_KIND_DIVA && n == 1);
    if (hooked) {
        const size_t n2 = (size_t)inst[0].nx * inst[0].ny;
        c->hook_buf.resize(4 * n2);
        hr.fn = t_hook;
        hr.user = t_hook_user;
        hr.nx = inst[0].nx;
        hr.ny = inst[0].ny;
        hr.d_out = c->d_out;
        hr.d_cbed = (double*)inst[0].c_bed;
        hr.d_uxb = inst[0].ux_b;
        hr.d_uyb = inst[0].uy_b;
        hr.h_cbed = host_cbed ? host_cbed : c->hook_buf.data();
        hr.h_uxb = c->hook_buf.data() + n2;
        hr.h_uyb = c->hook_buf.data() + 2 * n2;
        hr.h_prev = c->hook_buf.data() + 3 * n2;
        const int one = 1;
        CK(cudaMemcpyAsync(&c->d_out[0].defer, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
    }
    CK(cudaEventRecord(c->e0, c->stream));
    st = ygpu_launch_solver(c->device, c->stream, c->d_insts, n, *par, c->d_ctl, n_ctl, team_ctas, c->d_misc,
                            c->d_misc + 1, mapped ? c->d_map : nullptr, map_grid, c->use_graphs ? &c->graph : nullptr,
                            c->h_flags, c->check_every, hooked ? &hr : nullptr, c->spin_log2, c->cluster_ctas,
                            max_nu);
    if (st) return st;
    CK(cudaEventRecord(c->e1, c->stream));
    c->h_out.resize(n);
    CK(cudaMemcpyAsync(c->h_out.data(), c->d_out, sizeof(InstOut) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    int abort_flag = 0;
    CK(cudaMemcpyAsync(&abort_flag, c->d_misc + 1, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    ygpu_step_timing_flush();
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->e0, c->e1);
    int worst = YGPU_OK;
    for (int k = 0; k < n; k++) {
        const InstOut& o = c->h_out[k];
        int s_k = abort_flag ? YGPU_ERR_TIMEOUT : o.status;
        if (stats) {
            ygpu_stats& S = stats[k];
            S.ssa_iter_now = o.iter_now;
            S.ssa_lin_iter = o.lin_iter;
            S.ssa_lin_fail = o.lin_fail;
            S.ssa_lim_n = o.lim_n;
            S.ssa_resid = o.resid;
            S.lin_resid = o.lin_resid;
            S.outer_iter = o.outer_iter; S.active_cells = o.n_active;
            ygpu_lin_method_run_grid(par, inst[k].nx, inst[k].ny, &S.lin_solver_run, &S.lin_precond_run);
            S.status = s_k;
            S.device_ms = ms;
            for (int q = 0; q < 10; q++) S.phase_ms[q] = o.phase_ns[q] * 1e-6;
        }
        if (s_k < 0 && (worst >= 0 || s_k < worst)) worst = s_k;
        else if (worst >= 0 && s_k > worst) worst = s_k;
    }
    if (abort_flag) ygpu_set_error("a device-side wait hit its iteration limit (team barrier timeout)");
    return worst;
}

extern "C" int ygpu_solve_device(ygpu_ctx* c, int kind, const ygpu_dyn_par* par, const ygpu_fields* f,
                                 ygpu_stats* stats) {
    if (!c) { ygpu_set_error("context is NULL"); return YGPU_ERR_BAD_ARG; }
    return solve_batch(c, kind, par, 1, f, stats);
}

// Batches larger than one wave: continuous batching over a work queue. At most
// `max_active_unknowns` unknowns are on the GPU at once; each tick runs one
// Picard iteration (pre / Krylov / post) of the active instances, retires the
// finished ones and admits the next instances of the queue (largest first) into
// their scratch slots, so no instance waits for the slowest of the whole batch.
static int solve_queue(ygpu_ctx* c, int kind, const ygpu_dyn_par* par, int n, const ygpu_fields* inst,
                       ygpu_stats* stats) {
    const bool mixed = (par->precision == YGPU_PREC_MIXED);
    const bool block = ygpu_wants_block(*par);
    const bool ilu = ygpu_wants_ilu(*par);
    const size_t U = c->max_active_unknowns;
    std::vector<int> order(n);
    for (int k = 0; k < n; k++) order[k] = k;
    auto nu_of = [&](int k) { return (size_t)2 * inst[k].nx * inst[k].ny; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return (size_t)inst[a].nx * inst[a].ny * inst[a].nz > (size_t)inst[b].nx * inst[b].ny * inst[b].nz;
    });
    // slots: enough for the smallest instances to fill U, each sized for the largest
    size_t nu_min = nu_of(order[n - 1]), slot_bytes = 0;
    for (int k = 0; k < n; k++)
        slot_bytes = std::max(slot_bytes, al(ygpu_inst_scratch_bytes(inst[k].nx, inst[k].ny, inst[k].nz, mixed, block, ilu)));
    int n_slots = (int)std::min<size_t>((size_t)n, std::max<size_t>(1, U / std::max<size_t>(nu_min, 1) + 1));
    n_slots = std::min(n_slots, c->max_ctas > 0 ? c->max_ctas : 1);
    int st;
    if ((st = grow(&c->arena, &c->arena_cap, slot_bytes * (size_t)n_slots))) return st;
    const int cap = std::max(n, 2 * n_slots);
    if (c->insts_cap < cap) {
        cudaFree(c->d_insts);
        cudaFree(c->d_out);
        c->d_insts = nullptr;
        c->d_out = nullptr;
        CK(cudaMalloc((void**)&c->d_insts, sizeof(Inst) * (size_t)cap));
        CK(cudaMalloc((void**)&c->d_out, sizeof(InstOut) * (size_t)cap));
        c->insts_cap = cap;
    }
    const int n_ctl = c->max_ctas > 0 ? c->max_ctas : 1;
    if (c->ctl_cap < n_ctl) {
        cudaFree(c->d_ctl);
        c->d_ctl = nullptr;
        CK(cudaMalloc((void**)&c->d_ctl, sizeof(TeamCtl) * (size_t)n_ctl));
        c->ctl_cap = n_ctl;
    }
    const int map_need = 3 * n_ctl;
    if (c->map_cap < map_need) {
        cudaFree(c->d_map);
        c->d_map = nullptr;
        CK(cudaMalloc((void**)&c->d_map, sizeof(int) * (size_t)map_need));
        c->map_cap = map_need;
    }
    if ((st = ygpu_init_constants(c->device))) return st;
    // device layout: outputs per instance (caller order); active list, then admitted list
    InstOut* d_out = c->d_out;
    Inst* d_active = c->d_insts;
    Inst* d_new = c->d_insts + n_slots;
    int* d_done = c->d_misc;
    int* d_abort = c->d_misc + 1;
    CK(cudaMemsetAsync(d_out, 0, sizeof(InstOut) * (size_t)n, c->stream));
    CK(cudaMemsetAsync(c->d_misc, 0, 2 * sizeof(int), c->stream));
    CK(cudaMemsetAsync(c->d_ctl, 0, sizeof(TeamCtl) * (size_t)n_ctl, c->stream));
    if (c->spin_log2 > 0)
        CK(cudaMemset2DAsync(&c->d_ctl[0].spin_log2, sizeof(TeamCtl), c->spin_log2, 1, (size_t)n_ctl, c->stream));
    CK(cudaEventRecord(c->e0, c->stream));
    std::vector<int> slot_of(n, -1), free_slots;
    for (int k = n_slots - 1; k >= 0; k--) free_slots.push_back(k);
    std::vector<int> active;             // instance indices, largest first
    std::vector<Inst> h_active, h_new;
    c->h_out.resize(n);
    size_t active_nu = 0;
    int next = 0, abort_flag = 0;
    auto shape_of = [&](const std::vector<int>& ids, StepShape* sh) -> int {
        std::vector<size_t> nus;
        for (int k : ids) nus.push_back(nu_of(k));
        std::vector<int> map;
        int grid = 0;
        if (ids.size() > 1 && ygpu_plan_teams(c->max_ctas, (int)ids.size(), nus.data(), map, &grid, c->unknowns_per_cta)) {
            if (cudaMemcpyAsync(c->d_map, map.data(), sizeof(int) * map.size(), cudaMemcpyHostToDevice, c->stream) !=
                cudaSuccess)
                return YGPU_ERR_CUDA;
            // the host vector must outlive the copy
            if (cudaStreamSynchronize(c->stream) != cudaSuccess) return YGPU_ERR_CUDA;
            if (ygpu_step_shape_mapped(c->device, grid, c->d_map, sh) == YGPU_OK) {
                ygpu_step_shape_wide(sh, std::accumulate(nus.begin(), nus.end(), (size_t)0));
                return YGPU_OK;
            }
        }
        size_t mx = 0;
        for (size_t v : nus) mx = std::max(mx, v);
        int nt, tc;
        ygpu_choose_teams(c->max_ctas, (int)ids.size(), mx, &nt, &tc, c->unknowns_per_cta);
        const int r = ygpu_step_shape(c->device, nt, tc, sh);
        if (r == YGPU_OK) ygpu_step_shape_wide(sh, std::accumulate(nus.begin(), nus.end(), (size_t)0));
        return r;
    };
    while (next < n || !active.empty()) {
        // admit
        std::vector<int> adm;
        while (next < n && !free_slots.empty() &&
               ((active.empty() && adm.empty()) || active_nu + nu_of(order[next]) <= U)) {
            const int k = order[next++];
            const int s = free_slots.back();
            free_slots.pop_back();
            slot_of[k] = s;
            Inst I;
            ygpu_fill_inst(I, kind, &inst[k]);
            ygpu_inst_scratch_carve(I, c->arena + slot_bytes * (size_t)s, inst[k].nx, inst[k].ny, inst[k].nz, mixed,
                                    block, ilu);
            I.out = d_out + k;
            h_new.push_back(I);
            adm.push_back(k);
            active_nu += nu_of(k);
        }
        if (!adm.empty()) {
            CK(cudaMemcpyAsync(d_new, h_new.data(), sizeof(Inst) * h_new.size(), cudaMemcpyHostToDevice, c->stream));
            StepShape sh;
            if ((st = shape_of(adm, &sh))) return st;
            if ((st = ygpu_launch_step(YG_STEP_SETUP, c->stream, sh, d_new, (int)adm.size(), *par, c->d_ctl, d_done,
                                       d_abort)))
                return st;
            if (par->ssa_iter_max == 0 &&
                (st = ygpu_launch_step(YG_STEP_FINAL, c->stream, sh, d_new, (int)adm.size(), *par, c->d_ctl, d_done,
                                       d_abort)))
                return st;
            CK(cudaStreamSynchronize(c->stream));
            h_new.clear();
            for (int k : adm) active.push_back(k);
            std::stable_sort(active.begin(), active.end(), [&](int a, int b) { return nu_of(a) > nu_of(b); });
            h_active.clear();
            for (int k : active) {
                Inst I;
                ygpu_fill_inst(I, kind, &inst[k]);
                ygpu_inst_scratch_carve(I, c->arena + slot_bytes * (size_t)slot_of[k], inst[k].nx, inst[k].ny,
                                        inst[k].nz, mixed, block, ilu);
                I.out = d_out + k;
                h_active.push_back(I);
            }
            CK(cudaMemcpyAsync(d_active, h_active.data(), sizeof(Inst) * h_active.size(), cudaMemcpyHostToDevice,
                               c->stream));
        }
        if (active.empty()) continue;
        // one Picard iteration of every active instance
        StepShape sh;
        if ((st = shape_of(active, &sh))) return st;
        for (int step : {YG_STEP_PRE, YG_STEP_KRYLOV, YG_STEP_POST})
            if ((st = ygpu_launch_step(step, c->stream, sh, d_active, (int)active.size(), *par, c->d_ctl, d_done,
                                       d_abort)))
                return st;
        CK(cudaMemcpyAsync(c->h_out.data(), d_out, sizeof(InstOut) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaMemcpyAsync(c->h_flags + 1, d_abort, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        ygpu_step_timing_flush();
        abort_flag = c->h_flags[1];
        if (abort_flag) break;
        // retire
        std::vector<int> keep;
        for (int k : active) {
            if (c->h_out[k].done) {
                free_slots.push_back(slot_of[k]);
                active_nu -= nu_of(k);
            } else {
                keep.push_back(k);
            }
        }
        if (keep.size() != active.size()) {
            active.swap(keep);
            h_active.clear();
            for (int k : active) {
                Inst I;
                ygpu_fill_inst(I, kind, &inst[k]);
                ygpu_inst_scratch_carve(I, c->arena + slot_bytes * (size_t)slot_of[k], inst[k].nx, inst[k].ny,
                                        inst[k].nz, mixed, block, ilu);
                I.out = d_out + k;
                h_active.push_back(I);
            }
            if (!active.empty())
                CK(cudaMemcpyAsync(d_active, h_active.data(), sizeof(Inst) * h_active.size(), cudaMemcpyHostToDevice,
                                   c->stream));
        }
    }
    CK(cudaEventRecord(c->e1, c->stream));
    CK(cudaMemcpyAsync(c->h_out.data(), d_out, sizeof(InstOut) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->e0, c->e1);
    int worst = YGPU_OK;
    for (int k = 0; k < n; k++) {
        const InstOut& o = c->h_out[k];
        int s_k = abort_flag ? YGPU_ERR_TIMEOUT : o.status;
        if (stats) {
            ygpu_stats& S = stats[k];
            S.ssa_iter_now = o.iter_now;
            S.ssa_lin_iter = o.lin_iter;
            S.ssa_lin_fail = o.lin_fail;
            S.ssa_lim_n = o.lim_n;
            S.ssa_resid = o.resid;
            S.lin_resid = o.lin_resid;
            S.outer_iter = o.outer_iter; S.active_cells = o.n_active;
            ygpu_lin_method_run_grid(par, inst[k].nx, inst[k].ny, &S.lin_solver_run, &S.lin_precond_run);
            S.status = s_k;
            S.device_ms = ms;
            for (int q = 0; q < 10; q++) S.phase_ms[q] = o.phase_ns[q] * 1e-6;
        }
        if (s_k < 0 && (worst >= 0 || s_k < worst)) worst = s_k;
        else if (worst >= 0 && s_k > worst) worst = s_k;
    }
    if (abort_flag) ygpu_set_error("a device-side wait hit its iteration limit (team barrier timeout)");
    return worst;
}

extern "C" int ygpu_solve_batch_device(ygpu_ctx* c, int kind, const ygpu_dyn_par* par, int n_inst,
                                       const ygpu_fields* inst, ygpu_stats* stats) {
    if (!c) { ygpu_set_error("context is NULL"); return YGPU_ERR_BAD_ARG; }
    if (n_inst > 1 && c->max_active_unknowns > 0) {
        size_t total = 0;
        for (int k = 0; k < n_inst; k++) total += (size_t)2 * inst[k].nx * inst[k].ny;
        if (total > c->max_active_unknowns) {
            int st = ygpu_check_par(par);
            if (st) return st;
            if (kind != YGPU_KIND_SSA && kind != YGPU_KIND_DIVA) { ygpu_set_error("bad solver kind %d", kind); return YGPU_ERR_BAD_ARG; }
            for (int k = 0; k < n_inst; k++)
                if ((st = ygpu_fields_check(kind, &inst[k]))) return st;
            CK(cudaSetDevice(c->device));
            return solve_queue(c, kind, par, n_inst, inst, stats);
        }
    }
    return solve_batch(c, kind, par, n_inst, inst, stats);
}

// ---------------------------------------------------------------------------
// host-pointer drop-ins
// ---------------------------------------------------------------------------
namespace {
struct HostArg {
    void* host;          // host pointer
    size_t bytes;
    bool in, out;
    void* dev;
    size_t off;          // offset in the staging buffers
};

// Copies of many host segments, on several host threads when they are large
// (pieces of at most 4 MiB taken from a shared counter).
struct Seg {
    void* dst;
    const void* src;
    size_t n;
};

static void copy_segments(const std::vector<Seg>& segs) {
    size_t total = 0;
    for (const Seg& g : segs) total += g.n;
    unsigned hw = std::thread::hardware_concurrency();
    unsigned T = total >= ((size_t)32 << 20) ? std::min(16u, std::max(1u, hw)) : 1u;
    if (T <= 1) {
        for (const Seg& g : segs) memcpy(g.dst, g.src, g.n);
        return;
    }
    const size_t piece = (size_t)4 << 20;
    std::vector<Seg> pieces;
    for (const Seg& g : segs)
        for (size_t o = 0; o < g.n; o += piece)
            pieces.push_back({(char*)g.dst + o, (const char*)g.src + o, std::min(piece, g.n - o)});
    std::atomic<size_t> next(0);
    auto work = [&]() {
        for (size_t i; (i = next.fetch_add(1)) < pieces.size();)
            memcpy(pieces[i].dst, pieces[i].src, pieces[i].n);
    };
    std::vector<std::thread> th;
    for (unsigned t = 1; t < T; t++) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
}

// A copy list entry of the direct host<->device copies: one piece of at most
// YG_PIECE bytes of one array.
struct CopyPiece {
    const char* src;
    char* dst;
    unsigned long long n;
};
#define YG_PIECE (256u << 10)
// One CTA per piece (grid-stride over the list): 16-byte words where both
// addresses are 16-byte aligned, else 4-byte words (every array here holds
// 4- or 8-byte elements), then the tail bytes.
__global__ void __launch_bounds__(512) k_copy_pieces(const CopyPiece* __restrict__ list, int n) {
    for (int b = blockIdx.x; b < n; b += gridDim.x) {
        const CopyPiece q = list[b];
        unsigned long long done = 0;
        if ((((unsigned long long)q.src | (unsigned long long)q.dst) & 15ull) == 0) {
            const unsigned long long w = q.n / 16;
            const uint4* s = (const uint4*)q.src;
            uint4* d = (uint4*)q.dst;
            for (unsigned long long i = threadIdx.x; i < w; i += blockDim.x) d[i] = s[i];
            done = w * 16;
        } else if ((((unsigned long long)q.src | (unsigned long long)q.dst) & 3ull) == 0) {
            const unsigned long long w = q.n / 4;
            const unsigned* s = (const unsigned*)q.src;
            unsigned* d = (unsigned*)q.dst;
            for (unsigned long long i = threadIdx.x; i < w; i += blockDim.x) d[i] = s[i];
            done = w * 4;
        }
        for (unsigned long long i = done + threadIdx.x; i < q.n; i += blockDim.x) q.dst[i] = q.src[i];
    }
}

// Host staging of the host-pointer entries. The device buffer holds the arrays in
// the order in-only, in/out, out-only, then device-only scratch. Where the device
// reads and writes pageable host memory itself (cudaDevAttrPageableMemoryAccess,
// the coherent host-device link of Grace-based parts), one kernel gathers the
// inputs from the caller's arrays and one scatters the results back: no host copy
// at all. Elsewhere the arrays are packed into a pinned mirror: the inputs go up
// in one copy and the results come back in one.
struct Staging {
    std::vector<HostArg> args;
    size_t up = 0, down = 0, dend = 0, tot = 0;   // [0, up) goes up, [down, dend) comes back; scratch after
    bool direct = false;
    size_t add(void* h, size_t bytes, bool in, bool out) {
        args.push_back({h, bytes, in, out, nullptr, 0});
        return args.size() - 1;
    }
    // the pieces of the arrays of one direction, copied by one kernel on the stream
    int copy_direct(ygpu_ctx* c, bool to_device) {
        std::vector<CopyPiece> list;
        for (auto& a : args) {
            if (to_device ? !a.in : !a.out) continue;
            char* dev = c->fbuf + a.off;
            char* host = (char*)a.host;
            for (size_t o = 0; o < a.bytes; o += YG_PIECE) {
                const size_t n = std::min((size_t)YG_PIECE, a.bytes - o);
                list.push_back(to_device ? CopyPiece{host + o, dev + o, n} : CopyPiece{dev + o, host + o, n});
            }
        }
        if (list.empty()) return YGPU_OK;
        const size_t lb = list.size() * sizeof(CopyPiece);
        int st = grow(&c->dpieces, &c->dpieces_cap, lb);
        if (st) return st;
        // the list goes up from pageable memory: the call returns once it is staged
        CK(cudaMemcpyAsync(c->dpieces, list.data(), lb, cudaMemcpyHostToDevice, c->stream));
        const int grid = std::min((int)list.size(), 4 * std::max(c->sms, 1));
        k_copy_pieces<<<grid, 512, 0, c->stream>>>((const CopyPiece*)c->dpieces, (int)list.size());
        CK(cudaGetLastError());
        // the next call may rewrite the list: it waits for this copy first
        CK(cudaStreamSynchronize(c->stream));
        return YGPU_OK;
    }
    int upload(ygpu_ctx* c) {
        YgRange range("ygpu stage in");
        size_t off = 0;
        for (int cls = 0; cls < 4; cls++) {
            if (cls == 1) down = off;
            if (cls == 2) up = off;
            if (cls == 3) dend = off;
            for (auto& a : args) {
                const int ac = (a.in && !a.out) ? 0 : (a.in && a.out) ? 1 : a.out ? 2 : 3;
                if (ac != cls) continue;
                a.off = off;
                off += al(a.bytes);
            }
        }
        tot = off;
        int st = grow(&c->fbuf, &c->fbuf_cap, tot);
        if (st) return st;
        if (c->pageable < 0) {
            int v = 0;
            c->pageable = (cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccess, c->device) == cudaSuccess && v == 1)
                              ? 1 : 0;
            cudaGetLastError();
        }
        direct = (c->pageable == 1);
        if (direct) {
            for (auto& a : args) a.dev = c->fbuf + a.off;
            return copy_direct(c, true);
        }
        if (c->hbuf_cap < dend) {          // the pinned mirror leaves the scratch out
            if (c->hbuf) cudaFreeHost(c->hbuf);
            c->hbuf = nullptr;
            c->hbuf_cap = 0;
            if (cudaHostAlloc((void**)&c->hbuf, dend, cudaHostAllocDefault) != cudaSuccess) {
                cudaGetLastError();
                c->hbuf = nullptr;
                ygpu_set_error("pinned host allocation of %zu bytes failed", dend);
                return YGPU_ERR_NOMEM;
            }
            c->hbuf_cap = dend;
        }
        std::vector<Seg> segs;
        for (auto& a : args) {
            a.dev = c->fbuf + a.off;
            if (a.in) segs.push_back({c->hbuf + a.off, a.host, a.bytes});
        }
        copy_segments(segs);
        if (up) CK(cudaMemcpyAsync(c->fbuf, c->hbuf, up, cudaMemcpyHostToDevice, c->stream));
        return YGPU_OK;
    }
    int download(ygpu_ctx* c) {
        YgRange range("ygpu stage out");
        if (direct) return copy_direct(c, false);
        if (dend > down) CK(cudaMemcpyAsync(c->hbuf + down, c->fbuf + down, dend - down, cudaMemcpyDeviceToHost, c->stream));
        CK(cudaStreamSynchronize(c->stream));
        std::vector<Seg> segs;
        for (auto& a : args)
            if (a.out) segs.push_back({a.host, c->hbuf + a.off, a.bytes});
        copy_segments(segs);
        return YGPU_OK;
    }
};
}  // namespace

static bool any_null(std::initializer_list<const void*> ps) {
    for (const void* p : ps)
        if (!p) return true;
    return false;
}

extern "C" int ygpu_calc_velocity_ssa(double* ux_b, double* uy_b, double* taub_acx, double* taub_acy,
                                      double* visc_eff, double* visc_eff_int, int* ssa_mask_acx, int* ssa_mask_acy,
                                      double* ssa_err_acx, double* ssa_err_acy, int* ssa_iter_now, int* ssa_lin_iter,
                                      int* ssa_lin_fail, int* ssa_lim_n, double* beta, double* beta_acx,
                                      double* beta_acy, const double* c_bed, const double* f_slide,
                                      const double* taud_acx, const double* taud_acy, const double* taul_int_acx,
                                      const double* taul_int_acy, const double* H_ice, const double* f_ice,
                                      const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                                      const double* f_grnd_acy, const double* ATT, const double* zeta_aa,
                                      const double* z_sl, const double* z_bed, const double* z_srf, double dx,
                                      double dy, double n_glen, int nx, int ny, int nz, const ygpu_dyn_par* par) {
    if (nx < 3 || ny < 3 || nz < 2) { ygpu_set_error("grid too small: nx=%d ny=%d nz=%d", nx, ny, nz); return YGPU_ERR_BAD_ARG; }
    if (any_null({ux_b, uy_b, taub_acx, taub_acy, visc_eff, visc_eff_int, ssa_mask_acx, ssa_mask_acy, ssa_err_acx,
                  ssa_err_acy, ssa_iter_now, ssa_lin_iter, ssa_lin_fail, ssa_lim_n, beta, beta_acx, beta_acy, c_bed,
                  f_slide, taud_acx, taud_acy, taul_int_acx, taul_int_acy, H_ice, f_ice, H_grnd, f_grnd, f_grnd_acx,
                  f_grnd_acy, ATT, zeta_aa, z_sl, z_bed, z_srf})) {
        ygpu_set_error("NULL argument");
        return YGPU_ERR_BAD_ARG;
    }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)nx * ny * 8, b3 = b2 * nz, i2 = (size_t)nx * ny * 4;
    Staging S;
    size_t a_uxb = S.add(ux_b, b2, 1, 1), a_uyb = S.add(uy_b, b2, 1, 1);
    size_t a_tbx = S.add(taub_acx, b2, 1, 1), a_tby = S.add(taub_acy, b2, 1, 1);
    size_t a_v = S.add(visc_eff, b3, 1, 1), a_vi = S.add(visc_eff_int, b2, 0, 1);
    size_t a_mx = S.add(ssa_mask_acx, i2, 1, 0), a_my = S.add(ssa_mask_acy, i2, 1, 0);
    size_t a_ex = S.add(ssa_err_acx, b2, 0, 1), a_ey = S.add(ssa_err_acy, b2, 0, 1);
    size_t a_b = S.add(beta, b2, 1, 1), a_bx = S.add(beta_acx, b2, 1, 1), a_by = S.add(beta_acy, b2, 1, 1);
    size_t a_cb = S.add((void*)c_bed, b2, 1, 0), a_fs = S.add((void*)f_slide, b2, 1, 0);
    size_t a_tdx = S.add((void*)taud_acx, b2, 1, 0), a_tdy = S.add((void*)taud_acy, b2, 1, 0);
    size_t a_tlx = S.add((void*)taul_int_acx, b2, 1, 0), a_tly = S.add((void*)taul_int_acy, b2, 1, 0);
    size_t a_H = S.add((void*)H_ice, b2, 1, 0), a_fi = S.add((void*)f_ice, b2, 1, 0);
    size_t a_hg = S.add((void*)H_grnd, b2, 1, 0), a_fg = S.add((void*)f_grnd, b2, 1, 0);
    size_t a_fgx = S.add((void*)f_grnd_acx, b2, 1, 0), a_fgy = S.add((void*)f_grnd_acy, b2, 1, 0);
    size_t a_att = S.add((void*)ATT, b3, 1, 0), a_z = S.add((void*)zeta_aa, (size_t)nz * 8, 1, 0);
    size_t a_zsl = S.add((void*)z_sl, b2, 1, 0), a_zb = S.add((void*)z_bed, b2, 1, 0);
    size_t a_zs = S.add((void*)z_srf, b2, 1, 0);
    int st = S.upload(c);
    if (st) return st;
    auto d = [&](size_t k) { return (double*)S.args[k].dev; };
    ygpu_fields f;
    memset(&f, 0, sizeof(f));
    f.nx = nx; f.ny = ny; f.nz = nz; f.dx = dx; f.dy = dy; f.n_glen = n_glen;
    f.ux_b = d(a_uxb); f.uy_b = d(a_uyb); f.taub_acx = d(a_tbx); f.taub_acy = d(a_tby);
    f.visc_eff = d(a_v); f.visc_eff_int = d(a_vi);
    f.ssa_mask_acx = (int*)S.args[a_mx].dev; f.ssa_mask_acy = (int*)S.args[a_my].dev;
    f.ssa_err_acx = d(a_ex); f.ssa_err_acy = d(a_ey);
    f.beta = d(a_b); f.beta_acx = d(a_bx); f.beta_acy = d(a_by);
    f.c_bed = d(a_cb); f.f_slide = d(a_fs); f.taud_acx = d(a_tdx); f.taud_acy = d(a_tdy);
    f.taul_int_acx = d(a_tlx); f.taul_int_acy = d(a_tly); f.H_ice = d(a_H); f.f_ice = d(a_fi);
    f.H_grnd = d(a_hg); f.f_grnd = d(a_fg); f.f_grnd_acx = d(a_fgx); f.f_grnd_acy = d(a_fgy);
    f.ATT = d(a_att); f.zeta_aa = d(a_z); f.z_sl = d(a_zsl); f.z_bed = d(a_zb); f.z_srf = d(a_zs);
    ygpu_stats sts;
    memset(&sts, 0, sizeof(sts));
    st = solve_batch(c, YGPU_KIND_SSA, par, 1, &f, &sts);
    if (st == YGPU_ERR_CUDA || st == YGPU_ERR_NOMEM || st == YGPU_ERR_BAD_ARG) return st;
    int st2 = S.download(c);
    if (st2) return st2;
    *ssa_iter_now = sts.ssa_iter_now;
    *ssa_lin_iter = sts.ssa_lin_iter;
    *ssa_lin_fail = sts.ssa_lin_fail;
    *ssa_lim_n = sts.ssa_lim_n;
    return st;
}

extern "C" int ygpu_calc_velocity_diva(double* ux, double* uy, double* ux_bar, double* uy_bar, double* ux_b,
                                       double* uy_b, double* ux_i, double* uy_i, double* taub_acx, double* taub_acy,
                                       double* beta, double* beta_acx, double* beta_acy, double* beta_eff,
                                       double* visc_eff, double* visc_eff_int, double* duxdz, double* duydz,
                                       int* ssa_mask_acx, int* ssa_mask_acy, double* ssa_err_acx,
                                       double* ssa_err_acy, int* ssa_iter_now, int* ssa_lin_iter, int* ssa_lin_fail,
                                       int* ssa_lim_n, const double* c_bed, const double* f_slide,
                                       const double* taud_acx, const double* taud_acy, const double* taul_int_acx,
                                       const double* taul_int_acy, const double* H_ice, const double* f_ice,
                                       const double* H_grnd, const double* f_grnd, const double* f_grnd_acx,
                                       const double* f_grnd_acy, const double* ATT, const double* zeta_aa,
                                       const double* z_sl, const double* z_bed, const double* z_srf, double dx,
                                       double dy, double n_glen, int nx, int ny, int nz, const ygpu_dyn_par* par) {
    if (nx < 3 || ny < 3 || nz < 2) { ygpu_set_error("grid too small: nx=%d ny=%d nz=%d", nx, ny, nz); return YGPU_ERR_BAD_ARG; }
    if (any_null({ux, uy, ux_bar, uy_bar, ux_b, uy_b, ux_i, uy_i, taub_acx, taub_acy, beta, beta_acx, beta_acy,
                  beta_eff, visc_eff, visc_eff_int, duxdz, duydz, ssa_mask_acx, ssa_mask_acy, ssa_err_acx,
                  ssa_err_acy, ssa_iter_now, ssa_lin_iter, ssa_lin_fail, ssa_lim_n, c_bed, f_slide, taud_acx,
                  taud_acy, taul_int_acx, taul_int_acy, H_ice, f_ice, H_grnd, f_grnd, f_grnd_acx, f_grnd_acy, ATT,
                  zeta_aa, z_sl, z_bed, z_srf})) {
        ygpu_set_error("NULL argument");
        return YGPU_ERR_BAD_ARG;
    }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)nx * ny * 8, b3 = b2 * nz, i2 = (size_t)nx * ny * 4;
    Staging S;
    size_t a_ux = S.add(ux, b3, 0, 1), a_uy = S.add(uy, b3, 0, 1);
    size_t a_uxbar = S.add(ux_bar, b2, 1, 1), a_uybar = S.add(uy_bar, b2, 1, 1);
    size_t a_uxb = S.add(ux_b, b2, 1, 1), a_uyb = S.add(uy_b, b2, 1, 1);
    size_t a_uxi = S.add(ux_i, b3, 0, 1), a_uyi = S.add(uy_i, b3, 0, 1);
    size_t a_tbx = S.add(taub_acx, b2, 1, 1), a_tby = S.add(taub_acy, b2, 1, 1);
    size_t a_b = S.add(beta, b2, 1, 1), a_bx = S.add(beta_acx, b2, 1, 1), a_by = S.add(beta_acy, b2, 1, 1);
    size_t a_be = S.add(beta_eff, b2, 0, 1);
    size_t a_v = S.add(visc_eff, b3, 1, 1), a_vi = S.add(visc_eff_int, b2, 0, 1);
    size_t a_dx = S.add(duxdz, b3, 0, 1), a_dy = S.add(duydz, b3, 0, 1);
    size_t a_mx = S.add(ssa_mask_acx, i2, 1, 0), a_my = S.add(ssa_mask_acy, i2, 1, 0);
    size_t a_ex = S.add(ssa_err_acx, b2, 0, 1), a_ey = S.add(ssa_err_acy, b2, 0, 1);
    size_t a_cb = S.add((void*)c_bed, b2, 1, 0), a_fs = S.add((void*)f_slide, b2, 1, 0);
    size_t a_tdx = S.add((void*)taud_acx, b2, 1, 0), a_tdy = S.add((void*)taud_acy, b2, 1, 0);
    size_t a_tlx = S.add((void*)taul_int_acx, b2, 1, 0), a_tly = S.add((void*)taul_int_acy, b2, 1, 0);
    size_t a_H = S.add((void*)H_ice, b2, 1, 0), a_fi = S.add((void*)f_ice, b2, 1, 0);
    size_t a_hg = S.add((void*)H_grnd, b2, 1, 0), a_fg = S.add((void*)f_grnd, b2, 1, 0);
    size_t a_fgx = S.add((void*)f_grnd_acx, b2, 1, 0), a_fgy = S.add((void*)f_grnd_acy, b2, 1, 0);
    size_t a_att = S.add((void*)ATT, b3, 1, 0), a_z = S.add((void*)zeta_aa, (size_t)nz * 8, 1, 0);
    size_t a_zsl = S.add((void*)z_sl, b2, 1, 0), a_zb = S.add((void*)z_bed, b2, 1, 0);
    size_t a_zs = S.add((void*)z_srf, b2, 1, 0);
    int st = S.upload(c);
    if (st) return st;
    auto d = [&](size_t k) { return (double*)S.args[k].dev; };
    ygpu_fields f;
    memset(&f, 0, sizeof(f));
    f.nx = nx; f.ny = ny; f.nz = nz; f.dx = dx; f.dy = dy; f.n_glen = n_glen;
    f.ux = d(a_ux); f.uy = d(a_uy); f.ux_bar = d(a_uxbar); f.uy_bar = d(a_uybar);
    f.ux_b = d(a_uxb); f.uy_b = d(a_uyb); f.ux_i = d(a_uxi); f.uy_i = d(a_uyi);
    f.taub_acx = d(a_tbx); f.taub_acy = d(a_tby); f.beta = d(a_b); f.beta_acx = d(a_bx); f.beta_acy = d(a_by);
    f.beta_eff = d(a_be); f.visc_eff = d(a_v); f.visc_eff_int = d(a_vi); f.duxdz = d(a_dx); f.duydz = d(a_dy);
    f.ssa_mask_acx = (int*)S.args[a_mx].dev; f.ssa_mask_acy = (int*)S.args[a_my].dev;
    f.ssa_err_acx = d(a_ex); f.ssa_err_acy = d(a_ey);
    f.c_bed = d(a_cb); f.f_slide = d(a_fs); f.taud_acx = d(a_tdx); f.taud_acy = d(a_tdy);
    f.taul_int_acx = d(a_tlx); f.taul_int_acy = d(a_tly); f.H_ice = d(a_H); f.f_ice = d(a_fi);
    f.H_grnd = d(a_hg); f.f_grnd = d(a_fg); f.f_grnd_acx = d(a_fgx); f.f_grnd_acy = d(a_fgy);
    f.ATT = d(a_att); f.zeta_aa = d(a_z); f.z_sl = d(a_zsl); f.z_bed = d(a_zb); f.z_srf = d(a_zs);
    ygpu_stats sts;
    memset(&sts, 0, sizeof(sts));
    // with a neff hook the hook updates the caller's c_bed in place (as the
    // reference's c_bed argument of the hook), and the device copy follows it
    st = solve_batch(c, YGPU_KIND_DIVA, par, 1, &f, &sts, t_hook ? (double*)c_bed : nullptr);
    if (st == YGPU_ERR_CUDA || st == YGPU_ERR_NOMEM || st == YGPU_ERR_BAD_ARG) return st;
    int st2 = S.download(c);
    if (st2) return st2;
    *ssa_iter_now = sts.ssa_iter_now;
    *ssa_lin_iter = sts.ssa_lin_iter;
    *ssa_lin_fail = sts.ssa_lin_fail;
    *ssa_lim_n = sts.ssa_lim_n;
    return st;
}

// Batched solve on HOST arrays: every instance's fields (ygpu_fields of host
// pointers) go to the device, the batch runs as ygpu_solve_batch_device, and the
// in/out fields come back -- the arrays and directions of the single drop-ins.
extern "C" int ygpu_solve_batch_host(int kind, const ygpu_dyn_par* par, int n, const ygpu_fields* host,
                                     ygpu_stats* stats) {
    int st = ygpu_check_par(par);
    if (st) return st;
    if (kind != YGPU_KIND_SSA && kind != YGPU_KIND_DIVA) { ygpu_set_error("bad solver kind %d", kind); return YGPU_ERR_BAD_ARG; }
    if (n < 1 || !host) { ygpu_set_error("no instances"); return YGPU_ERR_BAD_ARG; }
    for (int k = 0; k < n; k++)
        if ((st = ygpu_fields_check(kind, &host[k]))) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const bool diva = (kind == YGPU_KIND_DIVA);
    Staging S;
    std::vector<std::vector<size_t>> ids(n);
    // (field offset in ygpu_fields, 3D?, in, out) in the order of the single drop-ins
    struct FD { size_t off; int dims; bool in, out, diva_only; };
#define FO(name) offsetof(ygpu_fields, name)
    static const FD tab[] = {
        {FO(ux), 3, false, true, true}, {FO(uy), 3, false, true, true},
        {FO(ux_bar), 2, true, true, true}, {FO(uy_bar), 2, true, true, true},
        {FO(ux_b), 2, true, true, false}, {FO(uy_b), 2, true, true, false},
        {FO(ux_i), 3, false, true, true}, {FO(uy_i), 3, false, true, true},
        {FO(taub_acx), 2, true, true, false}, {FO(taub_acy), 2, true, true, false},
        {FO(beta), 2, true, true, false}, {FO(beta_acx), 2, true, true, false}, {FO(beta_acy), 2, true, true, false},
        {FO(beta_eff), 2, false, true, true},
        {FO(visc_eff), 3, true, true, false}, {FO(visc_eff_int), 2, false, true, false},
        {FO(duxdz), 3, false, true, true}, {FO(duydz), 3, false, true, true},
        {FO(ssa_err_acx), 2, false, true, false}, {FO(ssa_err_acy), 2, false, true, false},
        {FO(ssa_mask_acx), -2, true, false, false}, {FO(ssa_mask_acy), -2, true, false, false},
        {FO(c_bed), 2, true, false, false}, {FO(f_slide), 2, true, false, false},
        {FO(taud_acx), 2, true, false, false}, {FO(taud_acy), 2, true, false, false},
        {FO(taul_int_acx), 2, true, false, false}, {FO(taul_int_acy), 2, true, false, false},
        {FO(H_ice), 2, true, false, false}, {FO(f_ice), 2, true, false, false},
        {FO(H_grnd), 2, true, false, false}, {FO(f_grnd), 2, true, false, false},
        {FO(f_grnd_acx), 2, true, false, false}, {FO(f_grnd_acy), 2, true, false, false},
        {FO(ATT), 3, true, false, false}, {FO(zeta_aa), 1, true, false, false},
        {FO(z_sl), 2, true, false, false}, {FO(z_bed), 2, true, false, false}, {FO(z_srf), 2, true, false, false},
    };
#undef FO
    const int nt = (int)(sizeof(tab) / sizeof(tab[0]));
    const bool hooked_cbed = (t_hook != nullptr && diva && n == 1);
    for (int k = 0; k < n; k++) {
        const ygpu_fields& h = host[k];
        const size_t b2 = (size_t)h.nx * h.ny * 8, b3 = b2 * h.nz, i2 = (size_t)h.nx * h.ny * 4;
        for (int q = 0; q < nt; q++) {
            void* ptr = *(void* const*)((const char*)&h + tab[q].off);
            if (!ptr || (tab[q].diva_only && !diva)) {
                ids[k].push_back((size_t)-1);
                continue;
            }
            const size_t bytes = tab[q].dims == 3 ? b3 : tab[q].dims == 2 ? b2 : tab[q].dims == -2 ? i2 : (size_t)h.nz * 8;
            // a single DIVA solve with a neff hook updates c_bed (as the drop-in does)
            const bool cbed_out = hooked_cbed && tab[q].off == offsetof(ygpu_fields, c_bed);
            ids[k].push_back(S.add(ptr, bytes, tab[q].in, tab[q].out || cbed_out));
        }
    }
    if ((st = S.upload(c))) return st;
    std::vector<ygpu_fields> dev(n);
    for (int k = 0; k < n; k++) {
        dev[k] = host[k];
        for (int q = 0; q < nt; q++) {
            void** slot = (void**)((char*)&dev[k] + tab[q].off);
            *slot = (ids[k][q] == (size_t)-1) ? nullptr : S.args[ids[k][q]].dev;
        }
    }
    st = ygpu_solve_batch_device(c, kind, par, n, dev.data(), stats);
    if (st == YGPU_ERR_CUDA || st == YGPU_ERR_NOMEM || st == YGPU_ERR_BAD_ARG) return st;
    int st2 = S.download(c);
    return st2 ? st2 : st;
}

extern "C" int ygpu_set_ssa_masks(int* mx, int* my, const int* mf, const double* f_ice, const double* f_grnd,
                                  int lateral_bc, int boundaries, int nx, int ny) {
    if (nx < 2 || ny < 2 || any_null({mx, my, mf, f_ice, f_grnd})) { ygpu_set_error("bad arguments"); return YGPU_ERR_BAD_ARG; }
    if (boundaries < 0 || boundaries > 6 || lateral_bc < 0 || lateral_bc > 3) { ygpu_set_error("bad code"); return YGPU_ERR_BAD_ARG; }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)nx * ny * 8, i2 = (size_t)nx * ny * 4;
    Staging S;
    size_t a_mx = S.add(mx, i2, 0, 1), a_my = S.add(my, i2, 0, 1), a_mf = S.add((void*)mf, i2, 1, 0);
    size_t a_fi = S.add((void*)f_ice, b2, 1, 0), a_fg = S.add((void*)f_grnd, b2, 1, 0);
    int st = S.upload(c);
    if (st) return st;
    st = ygpu_ssa_masks_device(c->stream, (int*)S.args[a_mx].dev, (int*)S.args[a_my].dev, (const int*)S.args[a_mf].dev,
                               (const double*)S.args[a_fi].dev, (const double*)S.args[a_fg].dev, lateral_bc,
                               boundaries, nx, ny);
    if (st) return st;
    return S.download(c);
}

extern "C" int ygpu_calc_dyn_inputs(const double* H_ice, const double* z_bed, const double* z_sl, double* f_ice,
                                    double* H_grnd, double* z_srf, double* f_grnd, double* f_grnd_acx,
                                    double* f_grnd_acy, int* mask_frnt, double* dzsdx, double* dzsdy,
                                    double* taud_acx, double* taud_acy, double* taul_int_acx, double* taul_int_acy,
                                    double dx, double grad_lim, double taud_lim, double rho_ice, double rho_sw,
                                    double g, int boundaries, int nx, int ny) {
    return ygpu_calc_dyn_inputs_bg(H_ice, z_bed, z_sl, f_ice, H_grnd, z_srf, f_grnd, f_grnd_acx, f_grnd_acy, mask_frnt,
                                   dzsdx, dzsdy, taud_acx, taud_acy, taul_int_acx, taul_int_acy, dx, grad_lim,
                                   taud_lim, rho_ice, rho_sw, g, 0.0, 0.0, boundaries, nx, ny);
}

extern "C" int ygpu_calc_dyn_inputs_bg(const double* H_ice, const double* z_bed, const double* z_sl, double* f_ice,
                                       double* H_grnd, double* z_srf, double* f_grnd, double* f_grnd_acx,
                                       double* f_grnd_acy, int* mask_frnt, double* dzsdx, double* dzsdy,
                                       double* taud_acx, double* taud_acy, double* taul_int_acx,
                                       double* taul_int_acy, double dx, double grad_lim, double taud_lim,
                                       double rho_ice, double rho_sw, double g, double slope_bg_x,
                                       double slope_bg_y, int boundaries, int nx, int ny) {
    if (nx < 3 || ny < 3 || !(dx > 0.0) || boundaries < 0 || boundaries > 6 || !isfinite(slope_bg_x) ||
        !isfinite(slope_bg_y) ||
        any_null({H_ice, z_bed, z_sl, f_ice, H_grnd, z_srf, f_grnd, f_grnd_acx, f_grnd_acy, mask_frnt, dzsdx, dzsdy,
                  taud_acx, taud_acy, taul_int_acx, taul_int_acy})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)nx * ny * 8, i2 = (size_t)nx * ny * 4;
    Staging S;
    size_t a_H = S.add((void*)H_ice, b2, 1, 0), a_zb = S.add((void*)z_bed, b2, 1, 0), a_zl = S.add((void*)z_sl, b2, 1, 0);
    size_t a_fi = S.add(f_ice, b2, 0, 1), a_hg = S.add(H_grnd, b2, 0, 1), a_zs = S.add(z_srf, b2, 0, 1);
    size_t a_fg = S.add(f_grnd, b2, 0, 1), a_fx = S.add(f_grnd_acx, b2, 0, 1), a_fy = S.add(f_grnd_acy, b2, 0, 1);
    size_t a_mf = S.add(mask_frnt, i2, 0, 1), a_dx = S.add(dzsdx, b2, 0, 1), a_dy = S.add(dzsdy, b2, 0, 1);
    size_t a_tx = S.add(taud_acx, b2, 0, 1), a_ty = S.add(taud_acy, b2, 0, 1);
    size_t a_lx = S.add(taul_int_acx, b2, 0, 1), a_ly = S.add(taul_int_acy, b2, 0, 1);
    int st = S.upload(c);
    if (st) return st;
    auto d = [&](size_t k) { return (double*)S.args[k].dev; };
    st = ygpu_dyn_inputs_device(c->stream, d(a_H), d(a_zb), d(a_zl), d(a_fi), d(a_hg), d(a_zs), d(a_fg), d(a_fx),
                                d(a_fy), (int*)S.args[a_mf].dev, d(a_dx), d(a_dy), d(a_tx), d(a_ty), d(a_lx), d(a_ly),
                                dx, grad_lim, taud_lim, rho_ice, rho_sw, g, boundaries, nx, ny, slope_bg_x,
                                slope_bg_y);
    if (st) return st;
    return S.download(c);
}

extern "C" int ygpu_calc_dyn_inputs_bg_device(ygpu_ctx* c, const double* H_ice, const double* z_bed,
                                              const double* z_sl, double* f_ice, double* H_grnd, double* z_srf,
                                              double* f_grnd, double* f_grnd_acx, double* f_grnd_acy, int* mask_frnt,
                                              double* dzsdx, double* dzsdy, double* taud_acx, double* taud_acy,
                                              double* taul_int_acx, double* taul_int_acy, double dx, double grad_lim,
                                              double taud_lim, double rho_ice, double rho_sw, double g,
                                              double slope_bg_x, double slope_bg_y, int boundaries, int nx, int ny) {
    if (!c || nx < 3 || ny < 3 || !(dx > 0.0) || boundaries < 0 || boundaries > 6 || !isfinite(slope_bg_x) ||
        !isfinite(slope_bg_y) ||
        any_null({H_ice, z_bed, z_sl, f_ice, H_grnd, z_srf, f_grnd, f_grnd_acx, f_grnd_acy, mask_frnt, dzsdx, dzsdy,
                  taud_acx, taud_acy, taul_int_acx, taul_int_acy})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    CK(cudaSetDevice(c->device));
    return ygpu_dyn_inputs_device(c->stream, H_ice, z_bed, z_sl, f_ice, H_grnd, z_srf, f_grnd, f_grnd_acx, f_grnd_acy,
                                  mask_frnt, dzsdx, dzsdy, taud_acx, taud_acy, taul_int_acx, taul_int_acy, dx,
                                  grad_lim, taud_lim, rho_ice, rho_sw, g, boundaries, nx, ny, slope_bg_x, slope_bg_y);
}

extern "C" int ygpu_set_ssa_masks_device(ygpu_ctx* c, int* ssa_mask_acx, int* ssa_mask_acy, const int* mask_frnt,
                                         const double* f_ice, const double* f_grnd, int lateral_bc, int boundaries,
                                         int nx, int ny) {
    if (!c || nx < 2 || ny < 2 || lateral_bc < 0 || lateral_bc > 3 || boundaries < 0 || boundaries > 6 ||
        any_null({ssa_mask_acx, ssa_mask_acy, mask_frnt, f_ice, f_grnd})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    CK(cudaSetDevice(c->device));
    return ygpu_ssa_masks_device(c->stream, ssa_mask_acx, ssa_mask_acy, mask_frnt, f_ice, f_grnd, lateral_bc,
                                 boundaries, nx, ny);
}

static int dyn_diag_check(const ygpu_dyn_diag* D, int bc) {
    if (!D || D->nx < 2 || D->ny < 2 || !(D->dx > 0.0) || !(D->dy > 0.0) || bc < 0 || bc > 6) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    if (any_null({D->ux_bar, D->uy_bar, D->ux_b, D->uy_b, D->taub_acx, D->taub_acy, D->taud_acx, D->taud_acy, D->H_ice,
                  D->f_ice, D->f_grnd, D->qq_acx, D->qq_acy, D->qq, D->qq_gl_acx, D->qq_gl_acy, D->taub, D->taud,
                  D->uxy_b, D->uxy_bar})) {
        ygpu_set_error("a required diagnostics array is NULL");
        return YGPU_ERR_BAD_ARG;
    }
    if (D->ux_i && (any_null({D->uy_i, D->zeta_aa, D->ux_i_bar, D->uy_i_bar}) || D->nz < 2)) {
        ygpu_set_error("ux_i needs uy_i, zeta_aa, ux_i_bar, uy_i_bar and nz >= 2");
        return YGPU_ERR_BAD_ARG;
    }
    if (D->uxy_i_bar && (!D->ux_i_bar || !D->uy_i_bar)) {
        ygpu_set_error("uxy_i_bar needs ux_i_bar and uy_i_bar");
        return YGPU_ERR_BAD_ARG;
    }
    if (D->ux && (any_null({D->uy, D->uxy, D->ux_s, D->uy_s, D->uxy_s, D->f_vbvs}) || D->nz < 1)) {
        ygpu_set_error("ux needs uy, uxy, ux_s, uy_s, uxy_s, f_vbvs and nz >= 1");
        return YGPU_ERR_BAD_ARG;
    }
    return YGPU_OK;
}

extern "C" int ygpu_calc_dyn_diagnostics_device(void* stream, const ygpu_dyn_diag* D, int boundaries) {
    int st = dyn_diag_check(D, boundaries);
    if (st) return st;
    return ygpu_dyn_diagnostics_device((cudaStream_t)stream, *D, boundaries);
}

// host arrays: in-only inputs, the depth averages in or out, every other output out
extern "C" int ygpu_calc_dyn_diagnostics(const ygpu_dyn_diag* H, int boundaries) {
    int st = dyn_diag_check(H, boundaries);
    if (st) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)H->nx * H->ny * 8, b3 = b2 * (size_t)(H->nz > 0 ? H->nz : 0);
    Staging S;
    ygpu_dyn_diag D = *H;
    std::vector<std::pair<size_t, const void**>> map;
    auto in = [&](const double* const* src, const double** dst, size_t bytes) {
        if (*src) map.push_back({S.add((void*)*src, bytes, 1, 0), (const void**)dst});
    };
    auto out = [&](double* const* src, double** dst, size_t bytes, bool also_in) {
        if (*src) map.push_back({S.add((void*)*src, bytes, also_in, 1), (const void**)dst});
    };
    in(&H->ux_bar, &D.ux_bar, b2); in(&H->uy_bar, &D.uy_bar, b2); in(&H->ux_b, &D.ux_b, b2); in(&H->uy_b, &D.uy_b, b2);
    in(&H->taub_acx, &D.taub_acx, b2); in(&H->taub_acy, &D.taub_acy, b2);
    in(&H->taud_acx, &D.taud_acx, b2); in(&H->taud_acy, &D.taud_acy, b2);
    in(&H->H_ice, &D.H_ice, b2); in(&H->f_ice, &D.f_ice, b2); in(&H->f_grnd, &D.f_grnd, b2);
    in(&H->ux_i, &D.ux_i, b3); in(&H->uy_i, &D.uy_i, b3); in(&H->zeta_aa, &D.zeta_aa, (size_t)H->nz * 8);
    in(&H->ux, &D.ux, b3); in(&H->uy, &D.uy, b3);
    const bool avg_out = (H->ux_i != nullptr);
    out(&H->ux_i_bar, &D.ux_i_bar, b2, !avg_out); out(&H->uy_i_bar, &D.uy_i_bar, b2, !avg_out);
    out(&H->qq_acx, &D.qq_acx, b2, false); out(&H->qq_acy, &D.qq_acy, b2, false); out(&H->qq, &D.qq, b2, false);
    out(&H->qq_gl_acx, &D.qq_gl_acx, b2, false); out(&H->qq_gl_acy, &D.qq_gl_acy, b2, false);
    out(&H->taub, &D.taub, b2, false); out(&H->taud, &D.taud, b2, false); out(&H->uxy_b, &D.uxy_b, b2, false);
    out(&H->uxy_i_bar, &D.uxy_i_bar, b2, false); out(&H->uxy_bar, &D.uxy_bar, b2, false);
    out(&H->uxy, &D.uxy, b3, false); out(&H->ux_s, &D.ux_s, b2, false); out(&H->uy_s, &D.uy_s, b2, false);
    out(&H->uxy_s, &D.uxy_s, b2, false); out(&H->f_vbvs, &D.f_vbvs, b2, false);
    if ((st = S.upload(c))) return st;
    for (auto& m : map) *m.second = S.args[m.first].dev;
    if ((st = ygpu_dyn_diagnostics_device(c->stream, D, boundaries))) return st;
    return S.download(c);
}

static int gradient_column_check(double* gx_c, double* gy_c, const double* gx, const double* gy, const double* f_ice,
                                 const int* ocn, int bc, int nx, int ny) {
    if (nx < 2 || ny < 2 || bc < 0 || bc > 6 || (size_t)nx * ny > (size_t)(1 << 28) ||
        any_null({gx_c, gy_c, gx, gy, f_ice, ocn})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    return YGPU_OK;
}

extern "C" int ygpu_calc_gradient_column_ac_device(void* stream, double* dvdx_c, double* dvdy_c, const double* dvdx,
                                                   const double* dvdy, const double* f_ice, const int* mask_ocn,
                                                   int boundaries, int nx, int ny) {
    int st = gradient_column_check(dvdx_c, dvdy_c, dvdx, dvdy, f_ice, mask_ocn, boundaries, nx, ny);
    if (st) return st;
    return ygpu_gradient_column_device((cudaStream_t)stream, dvdx_c, dvdy_c, dvdx, dvdy, f_ice, mask_ocn, boundaries,
                                       nx, ny);
}

extern "C" int ygpu_calc_gradient_column_ac(double* dvdx_c, double* dvdy_c, const double* dvdx, const double* dvdy,
                                            const double* f_ice, const int* mask_ocn, int boundaries, int nx,
                                            int ny) {
    int st = gradient_column_check(dvdx_c, dvdy_c, dvdx, dvdy, f_ice, mask_ocn, boundaries, nx, ny);
    if (st) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t n = (size_t)nx * ny, b2 = n * 8;
    Staging S;
    size_t a_gx = S.add((void*)dvdx, b2, 1, 0), a_gy = S.add((void*)dvdy, b2, 1, 0);
    size_t a_f = S.add((void*)f_ice, b2, 1, 0), a_o = S.add((void*)mask_ocn, n * 4, 1, 0);
    size_t a_cx = S.add(dvdx_c, b2, 0, 1), a_cy = S.add(dvdy_c, b2, 0, 1);
    if ((st = S.upload(c))) return st;
    auto d = [&](size_t a) { return (double*)S.args[a].dev; };
    if ((st = ygpu_gradient_column_device(c->stream, d(a_cx), d(a_cy), d(a_gx), d(a_gy), d(a_f),
                                          (const int*)S.args[a_o].dev, boundaries, nx, ny)))
        return st;
    return S.download(c);
}

static int jacobian_check(const ygpu_jvel* J, int bc, int terms) {
    if (!J || J->nx < 2 || J->ny < 2 || !(J->dx > 0.0) || !(J->dy > 0.0) || bc < 0 || bc > 6 || terms < 1 ||
        terms > 3 || (size_t)J->nx * J->ny > (size_t)(1 << 28) || J->nz_aa > 1000 || J->nz_ac > 1000) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    if (any_null({J->H_ice, J->f_ice, J->dzsdx, J->dzsdy, J->dzbdx, J->dzbdy})) {
        ygpu_set_error("H_ice, f_ice and the four column gradients are required");
        return YGPU_ERR_BAD_ARG;
    }
    if ((terms & YGPU_JAC_UXY) &&
        (J->nz_aa < 3 || any_null({J->ux, J->uy, J->zeta_aa, J->dxx, J->dxy, J->dxz, J->dyx, J->dyy, J->dyz}))) {
        ygpu_set_error("the ux/uy terms need ux, uy, zeta_aa, dxx ... dyz and nz_aa >= 3");
        return YGPU_ERR_BAD_ARG;
    }
    const bool dz_out = (terms & YGPU_JAC_UZ) || J->dzx || J->dzy || J->dzz;
    if (dz_out && (J->nz_ac < 1 || any_null({J->dzx, J->dzy, J->dzz}))) {
        ygpu_set_error("dzx, dzy, dzz go together and need nz_ac >= 1");
        return YGPU_ERR_BAD_ARG;
    }
    if ((terms & YGPU_JAC_UZ) && (J->nz_ac < 3 || any_null({J->uz, J->zeta_ac}))) {
        ygpu_set_error("the uz terms need uz, zeta_ac and nz_ac >= 3");
        return YGPU_ERR_BAD_ARG;
    }
    return YGPU_OK;
}

extern "C" int ygpu_calc_jacobian_vel_3D_device(void* stream, const ygpu_jvel* J, int boundaries, int terms) {
    int st = jacobian_check(J, boundaries, terms);
    if (st) return st;
    return ygpu_jacobian_device((cudaStream_t)stream, *J, boundaries, terms);
}

// host arrays: the inputs of the requested terms in, their components out
extern "C" int ygpu_calc_jacobian_vel_3D(const ygpu_jvel* H, int boundaries, int terms) {
    int st = jacobian_check(H, boundaries, terms);
    if (st) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t b2 = (size_t)H->nx * H->ny * 8;
    const bool uxy = terms & YGPU_JAC_UXY, uzt = terms & YGPU_JAC_UZ;
    const size_t ba = uxy ? b2 * (size_t)H->nz_aa : 0, bc3 = b2 * (size_t)(H->nz_ac > 0 ? H->nz_ac : 0);
    Staging S;
    ygpu_jvel D = *H;
    std::vector<std::pair<size_t, const void**>> map;
    auto in = [&](const double* src, const double** dst, size_t bytes) {
        map.push_back({S.add((void*)src, bytes, 1, 0), (const void**)dst});
    };
    auto out = [&](double* src, double** dst, size_t bytes) {
        map.push_back({S.add((void*)src, bytes, 0, 1), (const void**)dst});
    };
    in(H->H_ice, &D.H_ice, b2); in(H->f_ice, &D.f_ice, b2);
    in(H->dzsdx, &D.dzsdx, b2); in(H->dzsdy, &D.dzsdy, b2); in(H->dzbdx, &D.dzbdx, b2); in(H->dzbdy, &D.dzbdy, b2);
    if (uxy) {
        in(H->ux, &D.ux, ba); in(H->uy, &D.uy, ba); in(H->zeta_aa, &D.zeta_aa, (size_t)H->nz_aa * 8);
        out(H->dxx, &D.dxx, ba); out(H->dxy, &D.dxy, ba); out(H->dxz, &D.dxz, ba);
        out(H->dyx, &D.dyx, ba); out(H->dyy, &D.dyy, ba); out(H->dyz, &D.dyz, ba);
    }
    if (uzt) { in(H->uz, &D.uz, bc3); in(H->zeta_ac, &D.zeta_ac, (size_t)H->nz_ac * 8); }
    if (H->dzx) { out(H->dzx, &D.dzx, bc3); out(H->dzy, &D.dzy, bc3); out(H->dzz, &D.dzz, bc3); }
    if ((st = S.upload(c))) return st;
    for (auto& m : map) *m.second = S.args[m.first].dev;
    if ((st = ygpu_jacobian_device(c->stream, D, boundaries, terms))) return st;
    return S.download(c);
}

static int uz3d_check(const ygpu_uz3d* U, int bc, int method) {
    if (!U || U->nx < 2 || U->ny < 2 || !(U->dx > 0.0) || !(U->dy > 0.0) || bc < 0 || bc > 6 ||
        U->nz_aa < 2 || U->nz_aa > 1000 || U->nz_ac != U->nz_aa + 1 || (size_t)U->nx * U->ny > (size_t)(1 << 28)) {
        ygpu_set_error("bad arguments (nz_ac = nz_aa + 1, 2 <= nz_aa <= 1000)");
        return YGPU_ERR_BAD_ARG;
    }
    if (method < YGPU_UZ_AA || method > YGPU_UZ_FLUX) {
        ygpu_set_error("uz_method %d: 1 (uz_aa), 2 (uz_nodes), 3 (uz_jac) or 4 (uz_flux)", method);
        return YGPU_ERR_BAD_ARG;
    }
    if (method == YGPU_UZ_JAC && any_null({U->jac_dxx, U->jac_dyy})) {
        ygpu_set_error("uz_jac needs the Jacobian's jac_dxx and jac_dyy");
        return YGPU_ERR_BAD_ARG;
    }
    if (any_null({U->ux, U->uy, U->H_ice, U->f_ice, U->smb, U->bmb, U->dzbdt, U->dzsdt, U->dzsdx, U->dzsdy,
                  U->dzbdx, U->dzbdy, U->zeta_aa, U->zeta_ac, U->uz, U->uz_star})) {
        ygpu_set_error("a required vertical-velocity array is NULL");
        return YGPU_ERR_BAD_ARG;
    }
    if (method == YGPU_UZ_FLUX && any_null({U->ux_bar, U->uy_bar, U->dHidt_dyn, U->mask_kin})) {
        ygpu_set_error("uz_flux needs ux_bar, uy_bar, dHidt_dyn and mask_kin");
        return YGPU_ERR_BAD_ARG;
    }
    return YGPU_OK;
}

extern "C" int ygpu_calc_uz_3D_device(void* stream, const ygpu_uz3d* U, int boundaries, int method) {
    int st = uz3d_check(U, boundaries, method);
    if (st) return st;
    return ygpu_uz3d_device((cudaStream_t)stream, *U, boundaries, method);
}

extern "C" int ygpu_calc_uz_3D(const ygpu_uz3d* H, int boundaries, int method) {
    int st = uz3d_check(H, boundaries, method);
    if (st) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t n = (size_t)H->nx * H->ny, b2 = n * 8, ba = b2 * (size_t)H->nz_aa, bc3 = b2 * (size_t)H->nz_ac;
    Staging S;
    ygpu_uz3d D = *H;
    std::vector<std::pair<size_t, const void**>> map;
    auto in = [&](const void* src, const void** dst, size_t bytes) {
        map.push_back({S.add((void*)src, bytes, 1, 0), dst});
    };
    auto out = [&](double* src, double** dst, size_t bytes) {
        map.push_back({S.add((void*)src, bytes, 0, 1), (const void**)dst});
    };
    in(H->ux, (const void**)&D.ux, ba); in(H->uy, (const void**)&D.uy, ba);
    const double* const* f2[] = {&H->H_ice, &H->f_ice, &H->smb, &H->bmb, &H->dzbdt, &H->dzsdt,
                                 &H->dzsdx, &H->dzsdy, &H->dzbdx, &H->dzbdy};
    const double** d2[] = {&D.H_ice, &D.f_ice, &D.smb, &D.bmb, &D.dzbdt, &D.dzsdt,
                           &D.dzsdx, &D.dzsdy, &D.dzbdx, &D.dzbdy};
    for (int q = 0; q < 10; q++) in(*f2[q], (const void**)d2[q], b2);
    in(H->zeta_aa, (const void**)&D.zeta_aa, (size_t)H->nz_aa * 8);
    in(H->zeta_ac, (const void**)&D.zeta_ac, (size_t)H->nz_ac * 8);
    if (method == YGPU_UZ_FLUX) {
        in(H->ux_bar, (const void**)&D.ux_bar, b2); in(H->uy_bar, (const void**)&D.uy_bar, b2);
        in(H->dHidt_dyn, (const void**)&D.dHidt_dyn, b2); in(H->mask_kin, (const void**)&D.mask_kin, n * 4);
    }
    if (method == YGPU_UZ_JAC) {
        in(H->jac_dxx, (const void**)&D.jac_dxx, ba); in(H->jac_dyy, (const void**)&D.jac_dyy, ba);
    }
    out(H->uz, &D.uz, bc3); out(H->uz_star, &D.uz_star, bc3);
    if (H->uz_srf_err) out(H->uz_srf_err, &D.uz_srf_err, b2);
    if ((st = S.upload(c))) return st;
    for (auto& m : map) *m.second = S.args[m.first].dev;
    if ((st = ygpu_uz3d_device(c->stream, D, boundaries, method))) return st;
    return S.download(c);
}

static int strain3d_check(const ygpu_strain3d* S, int bc) {
    if (!S || S->nx < 2 || S->ny < 2 || !(S->dx > 0.0) || !(S->dy > 0.0) || bc < 0 || bc > 6 ||
        S->nz_aa < 2 || S->nz_aa > 1000 || S->nz_ac != S->nz_aa + 1 || (size_t)S->nx * S->ny > (size_t)(1 << 28) ||
        !(S->de_max >= 0.0)) {
        ygpu_set_error("bad arguments (nz_ac = nz_aa + 1, 2 <= nz_aa <= 1000, de_max >= 0)");
        return YGPU_ERR_BAD_ARG;
    }
    if (any_null({S->dxx, S->dxy, S->dxz, S->dyx, S->dyy, S->dyz, S->dzx, S->dzy, S->H_ice, S->f_ice, S->f_grnd,
                  S->zeta_aa, S->zeta_ac, S->s_dxx, S->s_dyy, S->s_dxy, S->s_dxz, S->s_dyz, S->s_de, S->s_div,
                  S->s_f_shear})) {
        ygpu_set_error("a required strain-rate array is NULL");
        return YGPU_ERR_BAD_ARG;
    }
    return YGPU_OK;
}

extern "C" int ygpu_calc_strain_rate_tensor_device(void* stream, const ygpu_strain3d* S, int boundaries) {
    int st = strain3d_check(S, boundaries);
    if (st) return st;
    return ygpu_strain3d_device((cudaStream_t)stream, *S, boundaries);
}

extern "C" int ygpu_calc_strain_rate_tensor(const ygpu_strain3d* H, int boundaries) {
    int st = strain3d_check(H, boundaries);
    if (st) return st;
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t n = (size_t)H->nx * H->ny, b2 = n * 8, ba = b2 * (size_t)H->nz_aa, bc3 = b2 * (size_t)H->nz_ac;
    Staging Sg;
    ygpu_strain3d D = *H;
    std::vector<std::pair<size_t, const void**>> map;
    auto in = [&](const void* src, const void** dst, size_t bytes) {
        map.push_back({Sg.add((void*)src, bytes, 1, 0), dst});
    };
    auto out = [&](double* src, double** dst, size_t bytes) {
        if (src) map.push_back({Sg.add((void*)src, bytes, 0, 1), (const void**)dst});
    };
    const double* const* f3[] = {&H->dxx, &H->dxy, &H->dxz, &H->dyx, &H->dyy, &H->dyz};
    const double** d3[] = {&D.dxx, &D.dxy, &D.dxz, &D.dyx, &D.dyy, &D.dyz};
    for (int q = 0; q < 6; q++) in(*f3[q], (const void**)d3[q], ba);
    in(H->dzx, (const void**)&D.dzx, bc3); in(H->dzy, (const void**)&D.dzy, bc3);
    in(H->H_ice, (const void**)&D.H_ice, b2); in(H->f_ice, (const void**)&D.f_ice, b2);
    in(H->f_grnd, (const void**)&D.f_grnd, b2);
    in(H->zeta_aa, (const void**)&D.zeta_aa, (size_t)H->nz_aa * 8);
    in(H->zeta_ac, (const void**)&D.zeta_ac, (size_t)H->nz_ac * 8);
    double* const o3h[] = {H->s_dxx, H->s_dyy, H->s_dxy, H->s_dxz, H->s_dyz, H->s_de, H->s_div, H->s_f_shear};
    double** o3d[] = {&D.s_dxx, &D.s_dyy, &D.s_dxy, &D.s_dxz, &D.s_dyz, &D.s_de, &D.s_div, &D.s_f_shear};
    for (int q = 0; q < 8; q++) out(o3h[q], o3d[q], ba);
    double* const o2h[] = {H->a_dxx, H->a_dyy, H->a_dxy, H->a_dxz, H->a_dyz, H->a_de, H->a_div, H->a_f_shear,
                           H->eps_eig_1, H->eps_eig_2};
    double** o2d[] = {&D.a_dxx, &D.a_dyy, &D.a_dxy, &D.a_dxz, &D.a_dyz, &D.a_de, &D.a_div, &D.a_f_shear,
                      &D.eps_eig_1, &D.eps_eig_2};
    for (int q = 0; q < 10; q++) out(o2h[q], o2d[q], b2);
    if ((st = Sg.upload(c))) return st;
    for (auto& m : map) *m.second = Sg.args[m.first].dev;
    if ((st = ygpu_strain3d_device(c->stream, D, boundaries))) return st;
    return Sg.download(c);
}

extern "C" int ygpu_calc_advec2D_impl_lis(double* dvdt, const double* var, const double* ux, const double* uy,
                                          const double* var_dot, const int* mask_ice, const double* var_ref,
                                          double dx, double dy, double dt, int boundaries, int nx, int ny,
                                          int* lin_iter, int* lin_status) {
    if (nx < 3 || ny < 3 || !(dx > 0.0) || !(dy > 0.0) || !(dt > 0.0) || boundaries < 0 || boundaries > 7 ||
        (size_t)nx * ny > (size_t)(1 << 28) ||
        any_null({dvdt, var, ux, uy, var_dot, mask_ice, var_ref, lin_iter, lin_status})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    const size_t n = (size_t)nx * ny, b2 = n * 8;
    Staging S;
    size_t a_v = S.add((void*)var, b2, 1, 0), a_ux = S.add((void*)ux, b2, 1, 0), a_uy = S.add((void*)uy, b2, 1, 0);
    size_t a_f = S.add((void*)var_dot, b2, 1, 0), a_m = S.add((void*)mask_ice, n * 4, 1, 0);
    size_t a_r = S.add((void*)var_ref, b2, 1, 0), a_d = S.add(dvdt, b2, 0, 1);
    size_t a_w = S.add(nullptr, b2 * 16, 0, 0);
    if (c->ctl_cap < 1) {
        CK(cudaMalloc((void**)&c->d_ctl, sizeof(TeamCtl)));
        c->ctl_cap = 1;
    }
    int st = S.upload(c);
    if (st) return st;
    int nct = (int)((n + 2 * YG_BLOCK - 1) / (2 * YG_BLOCK));
    if (nct > c->adv_max_ctas) nct = c->adv_max_ctas;
    if (nct > YG_MAX_TEAM_CTAS) nct = YG_MAX_TEAM_CTAS;
    if (nct < 1) nct = 1;
    auto d = [&](size_t k) { return (double*)S.args[k].dev; };
    st = ygpu_launch_advect(c->stream, nx, ny, boundaries, dx, dy, dt, d(a_v), d(a_ux), d(a_uy), d(a_f), d(a_r),
                            (const int*)S.args[a_m].dev, d(a_d), d(a_w), c->d_misc + 2, c->d_miscd, c->d_ctl,
                            c->d_misc + 1, nct);
    if (st) return st;
    int outi[2];
    CK(cudaMemcpyAsync(outi, c->d_misc + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    st = S.download(c);
    if (st) return st;
    *lin_iter = outi[0];
    *lin_status = outi[1];
    return outi[1] < 0 ? outi[1] : YGPU_OK;
}

// device arrays on a context's stream; scratch from the context's arena;
// synchronises to return the iteration count and status
extern "C" int ygpu_advec2D_impl_lis_device(ygpu_ctx* c, double* dvdt, const double* var, const double* ux,
                                            const double* uy, const double* var_dot, const int* mask_ice,
                                            const double* var_ref, double dx, double dy, double dt, int boundaries,
                                            int nx, int ny, int* lin_iter, int* lin_status) {
    if (!c || nx < 3 || ny < 3 || !(dx > 0.0) || !(dy > 0.0) || !(dt > 0.0) || boundaries < 0 || boundaries > 7 ||
        (size_t)nx * ny > (size_t)(1 << 28) ||
        any_null({dvdt, var, ux, uy, var_dot, mask_ice, var_ref, lin_iter, lin_status})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    CK(cudaSetDevice(c->device));
    const size_t n = (size_t)nx * ny;
    int st = grow(&c->arena, &c->arena_cap, n * 8 * 16);
    if (st) return st;
    if (c->ctl_cap < 1) {
        CK(cudaMalloc((void**)&c->d_ctl, sizeof(TeamCtl)));
        c->ctl_cap = 1;
    }
    int nct = (int)((n + 2 * YG_BLOCK - 1) / (2 * YG_BLOCK));
    if (nct > c->adv_max_ctas) nct = c->adv_max_ctas;
    if (nct > YG_MAX_TEAM_CTAS) nct = YG_MAX_TEAM_CTAS;
    if (nct < 1) nct = 1;
    st = ygpu_launch_advect(c->stream, nx, ny, boundaries, dx, dy, dt, var, ux, uy, var_dot, var_ref, mask_ice, dvdt,
                            (double*)c->arena, c->d_misc + 2, c->d_miscd, c->d_ctl, c->d_misc + 1, nct);
    if (st) return st;
    int outi[2];
    CK(cudaMemcpyAsync(outi, c->d_misc + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaStreamSynchronize(c->stream));
    *lin_iter = outi[0];
    *lin_status = outi[1];
    return outi[1] < 0 ? outi[1] : YGPU_OK;
}

extern "C" int ygpu_linear_solver_matrix_solve(int nmax, const int* a_ptr, const int* a_index, const double* a_value,
                                               const double* b_value, double* x_value, const char* lis_opt,
                                               int* lin_iter, int* status, double* L2_rel_norm) {
    if (nmax < 1 || any_null({a_ptr, a_index, a_value, b_value, x_value, lin_iter, status, L2_rel_norm})) {
        ygpu_set_error("bad arguments");
        return YGPU_ERR_BAD_ARG;
    }
    ygpu_dyn_par p;
    ygpu_dyn_par_defaults(&p);
    int st = ygpu_parse_lis_opt(lis_opt ? lis_opt : "", &p);
    if (st) return st;
    int nnz = a_ptr[nmax] - 1;
    if (nnz < 0 || a_ptr[0] != 1) { ygpu_set_error("a_ptr must be 1-based CSR"); return YGPU_ERR_BAD_ARG; }
    ygpu_ctx* c = default_ctx();
    if (!c) return YGPU_ERR_CUDA;
    // 0-based copies on the host (the Fortran arrays are 1-based)
    std::vector<int> ptr0(nmax + 1), idx0(nnz);
    for (int k = 0; k <= nmax; k++) ptr0[k] = a_ptr[k] - 1;
    for (int k = 0; k < nnz; k++) {
        idx0[k] = a_index[k] - 1;
        if (idx0[k] < 0 || idx0[k] >= nmax) { ygpu_set_error("column index out of range at %d", k); return YGPU_ERR_BAD_ARG; }
    }
    Staging S;
    size_t a_p = S.add(ptr0.data(), (size_t)(nmax + 1) * 4, 1, 0), a_i = S.add(idx0.data(), (size_t)nnz * 4, 1, 0);
    size_t a_v = S.add((void*)a_value, (size_t)nnz * 8, 1, 0), a_b = S.add((void*)b_value, (size_t)nmax * 8, 1, 0);
    size_t a_x = S.add(x_value, (size_t)nmax * 8, 1, 1);
    std::vector<double> dummy(1);
    size_t a_w = S.add(nullptr, (size_t)nmax * 8 * 12, 0, 0);
    if (c->ctl_cap < 1) {
        CK(cudaMalloc((void**)&c->d_ctl, sizeof(TeamCtl)));
        c->ctl_cap = 1;
    }
    st = S.upload(c);
    if (st) return st;
    int nct = (nmax + 2 * YG_BLOCK - 1) / (2 * YG_BLOCK);
    if (nct > c->csr_max_ctas) nct = c->csr_max_ctas;
    if (nct > YG_MAX_TEAM_CTAS) nct = YG_MAX_TEAM_CTAS;
    if (nct < 1) nct = 1;
    int method = p.lin_solver == YGPU_LIN_BICGSTAB ? YGPU_LIN_BICGSTAB : YGPU_LIN_CG;
    st = ygpu_launch_csr(c->stream, nmax, (const int*)S.args[a_p].dev, (const int*)S.args[a_i].dev,
                         (const double*)S.args[a_v].dev, (const double*)S.args[a_b].dev, (double*)S.args[a_x].dev,
                         (double*)S.args[a_w].dev, method, p.lin_precond, p.lin_maxiter, p.lin_tol,
                         p.lin_initx_zeros, c->d_misc + 2, c->d_miscd, c->d_ctl, c->d_misc + 1, nct);
    if (st) return st;
    int outi[2];
    double outd;
    CK(cudaMemcpyAsync(outi, c->d_misc + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CK(cudaMemcpyAsync(&outd, c->d_miscd, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    st = S.download(c);
    if (st) return st;
    *lin_iter = outi[0];
    *status = outi[1];
    *L2_rel_norm = outd;
    return outi[1];
}
